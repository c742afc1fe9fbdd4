"""aerojax_gb300: GB300-native (sm_103a) projection-method Navier-Stokes step.

Drop-in replacements, on torch CUDA tensors, for the hot path of AeroJAX:
``step_pure``, the GUI step ``StepHandler._step``, ``poisson_multigrid`` /
``poisson_multigrid_mac``, ``rk_step_unified`` / ``rk_step_unified_mac``,
``constant_smagorinsky`` / ``dynamic_smagorinsky`` and
``compute_cfl_timestep``.  All compute runs in libaerojax_gb300.so (C ABI in
include/aerojax_gb300.h); build it with ``python -m aerojax_gb300.build``.
"""
from .params import GridParams, SimState, StepConfig, compute_eps_multiplier, get_re_parameters
from .solver import (Plan, StepHandler, compute_cfl_timestep, constant_smagorinsky,
                     diagnostics, dynamic_smagorinsky, get_plan, make_geometry, poisson_multigrid,
                     post_step,
                     poisson_multigrid_converge, poisson_multigrid_mac, rk_step_unified,
                     rk_step_unified_mac, run_step, run_step_host, step_pure)

__all__ = [
    "GridParams", "SimState", "StepConfig", "compute_eps_multiplier", "get_re_parameters",
    "Plan", "StepHandler", "compute_cfl_timestep", "constant_smagorinsky", "diagnostics",
    "post_step",
    "dynamic_smagorinsky",
    "get_plan", "make_geometry", "poisson_multigrid", "poisson_multigrid_converge",
    "poisson_multigrid_mac", "rk_step_unified", "rk_step_unified_mac", "run_step",
    "run_step_host", "step_pure",
]
