"""Python host API with the reference's call signatures, on torch CUDA tensors.

Every function here enqueues work through the C ABI of libaerojax_gb300.so on
the current torch CUDA stream; tensors never leave the device and nothing
falls back to the CPU.  Reference counterparts:

  step_pure                    solver/pure_functions/step.py:49-467
  StepHandler._step            solver/simulation/step_handlers.py:296-301
  poisson_multigrid(_mac)      pressure_solvers/multigrid_solver.py:55-241,
                               pressure_solvers/multigrid_solver_mac.py:59-246
  rk_step_unified(_mac)        advection_schemes/rk3_simple_new.py:175-358,
                               advection_schemes/rk3_mac.py:220-504
  constant/dynamic_smagorinsky solver/les_models.py:79-200
  compute_cfl_timestep         timestepping/cfl_adaptive_dt.py:6-71
"""
from __future__ import annotations

import ctypes
from dataclasses import replace
from typing import Optional, Tuple

import torch

from . import _lib
from ._lib import AjStats, AjStepParams, check, lib
from .params import SimState, StepConfig


# ----------------------------------------------------------------- plumbing
def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _f32(t, name, shape=None, device=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch CUDA tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must live on a CUDA device (no CPU path exists)")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return t


def warm_mode(w) -> int:
    """StepConfig.warm_start -> AJ_WARM_*: False 0 (zero guess), True 1
    (p_guess), "extrapolate" 2 (the workspace's last two solutions)."""
    if isinstance(w, str):
        if w != "extrapolate":
            raise ValueError(f"warm_start={w!r}: expected a bool or 'extrapolate'")
        return 2
    return int(bool(w))


def make_params(cfg: StepConfig) -> AjStepParams:
    p = AjStepParams()
    p.nx, p.ny = cfg.nx, cfg.ny
    p.grid_type = _lib.GRID[cfg.grid_type]
    p.flow_type = _lib.FLOW[cfg.flow_type]
    p.variant = _lib.VARIANT[cfg.variant]
    p.les_model = _lib.LES[cfg.les_model] if cfg.use_les else 0
    p.advection = _lib.ADV[cfg.advection_scheme]
    p.mg_mode = _lib.MG[cfg.mg_mode]
    p.fast_mode = int(cfg.fast_mode)
    p.slip_walls = int(cfg.slip_walls)
    p.v_cycles = cfg.v_cycles
    p.levels = cfg.levels
    p.max_cycles = cfg.max_cycles
    p.has_sdf = int(cfg.has_sdf)
    p.cfl_dt = int(cfg.cfl_dt)
    p.warm_start = warm_mode(cfg.warm_start)
    p.nn_factor = int(cfg.nn_factor)
    p.dx, p.dy = cfg.dx, cfg.dy
    p.dt = cfg.dt
    p.dt_correction = cfg.dt_correction
    p.nu, p.U_inf, p.brinkman_eta = cfg.nu, cfg.U_inf, cfg.brinkman_eta
    p.smagorinsky_constant = cfg.smagorinsky_constant
    p.nu_hyper_ratio = cfg.nu_hyper_ratio
    p.mg_tolerance = cfg.mg_tolerance
    p.mg_rtol = cfg.mg_rtol
    p.cfl_target, p.dt_min, p.dt_max = cfg.cfl_target, cfg.dt_min, cfg.dt_max
    p.les_delta = cfg.les_delta
    return p


class Plan:
    """A device workspace sized for one StepConfig, prepared for one geometry.

    The workspace is allocated once (torch caching allocator) and re-used by
    every call; aj_prepare re-runs only when the mask/sdf tensors change."""

    def __init__(self, cfg: StepConfig, device):
        self.cfg = cfg
        self.params = make_params(cfg)
        L = lib()
        check("aj_check_params", L.aj_check_params(ctypes.byref(self.params)))
        self.nbytes = int(L.aj_workspace_size(ctypes.byref(self.params)))
        if self.nbytes == 0:
            raise ValueError("aj_workspace_size rejected the configuration")
        self.ws = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        if self.ws.data_ptr() % 256:
            raise RuntimeError("workspace is not 256-byte aligned")
        self.stats_buf = torch.zeros(_lib.STATS_BYTES, dtype=torch.uint8, device=device)
        self._geom_key = None

    def prepare(self, mask: torch.Tensor, sdf: Optional[torch.Tensor] = None, stream=None):
        key = (mask.data_ptr(), mask._version, None if sdf is None else (sdf.data_ptr(), sdf._version))
        if key == self._geom_key:
            return
        check("aj_prepare", lib().aj_prepare(ctypes.byref(self.params), mask.data_ptr(), _ptr(sdf),
                                             self.ws.data_ptr(), self.nbytes, _stream(stream)))
        self._geom_key = key

    def stats(self) -> dict:
        """Reads the device statistics of the last call (synchronises)."""
        raw = bytes(self.stats_buf.cpu().numpy().tobytes())
        s = AjStats.from_buffer_copy(raw)
        return {"cycles": s.cycles, "converged": bool(s.converged), "err": s.err,
                "err_name": _lib.STATUS_NAMES.get(s.err, s.err), "rel_residual": s.rel_residual,
                "rhs_norm": s.rhs_norm, "dt": s.dt, "abs_residual_sq": s.abs_residual_sq}


_PLANS: dict = {}


def get_plan(cfg: StepConfig, device) -> Plan:
    key = (repr(replace(cfg, dt=0.0, nn_model=None)), str(device))
    plan = _PLANS.get(key)
    if plan is None:
        plan = Plan(cfg, device)
        _PLANS[key] = plan
    return plan


def run_step(plan: Plan, u, v, mask, p_guess=None, out=None, stream=None, dt=None):
    """One projection step through aj_step; returns (u_new, v_new, p)."""
    cfg = plan.cfg
    if dt is not None and not cfg.cfl_dt and dt != plan.params.dt:
        plan.params.dt = float(dt)
    if out is None:
        out = (torch.empty_like(u), torch.empty_like(v),
               torch.empty((cfg.nx, cfg.ny), dtype=torch.float32, device=u.device))
    uo, vo, po = out
    check("aj_step", lib().aj_step(ctypes.byref(plan.params), u.data_ptr(), v.data_ptr(),
                                   mask.data_ptr(), _ptr(p_guess), uo.data_ptr(), vo.data_ptr(),
                                   po.data_ptr(), plan.ws.data_ptr(), plan.nbytes,
                                   plan.stats_buf.data_ptr(), _stream(stream)))
    return uo, vo, po


def run_step_host(plan: Plan, h_u, h_v, mask, h_p=None, h_out=None, net=None, stream=None):
    """One step with the fields in pinned HOST memory (aj_step_host): the
    uploads, the step (the learned warm start with ``net``) and the downloads
    in one graph launch, the pressure's transfers overlapped with the
    predictor and the correction.  Returns (u_new, v_new, p) as host tensors
    (``h_out`` if given)."""
    cfg = plan.cfg
    mac = cfg.grid_type == "mac"
    nu = (cfg.nx + 1) * cfg.ny if mac else cfg.nx * cfg.ny
    nv = cfg.nx * (cfg.ny + 1) if mac else cfg.nx * cfg.ny
    n = nu + nv + cfg.nx * cfg.ny
    dev = plan.ws.device
    stage = getattr(plan, "_host_stage", None)
    if stage is None or stage[0].numel() != n:
        stage = (torch.empty(n, dtype=torch.float32, device=dev),
                 torch.empty(n, dtype=torch.float32, device=dev))
        plan._host_stage = stage
    if h_out is None:
        h_out = (torch.empty_like(h_u).pin_memory(), torch.empty_like(h_v).pin_memory(),
                 torch.empty((cfg.nx, cfg.ny), dtype=torch.float32).pin_memory())
    # the copies are recorded into the step's graph: every host buffer must be
    # page-locked
    named = [(h_u, "h_u"), (h_v, "h_v"), (h_out[0], "h_out[0]"), (h_out[1], "h_out[1]"),
             (h_out[2], "h_out[2]")]
    if h_p is not None:
        named.append((h_p, "h_p"))
    for t, name in named:
        if t.is_cuda or not t.is_pinned():
            raise ValueError(f"{name} must be a pinned host tensor")
    packed = master = None
    if net is not None:   # an aerojax_gb300.nn.WarmStartNet (its packed BF16 weights current)
        packed, master = net.packed.data_ptr(), net.master.data_ptr()
    check("aj_step_host", lib().aj_step_host(
        ctypes.byref(plan.params), h_u.data_ptr(), h_v.data_ptr(), mask.data_ptr(), _ptr(h_p),
        h_out[0].data_ptr(), h_out[1].data_ptr(), h_out[2].data_ptr(), stage[0].data_ptr(),
        stage[1].data_ptr(), packed, master, plan.ws.data_ptr(), plan.nbytes,
        plan.stats_buf.data_ptr(), _stream(stream)))
    return h_out


# ----------------------------------------------------------------- step_pure
def step_pure(state: SimState, mask, sdf, dx, dy, nu, U_inf, use_les=False,
              smagorinsky_constant=0.1, weno_epsilon=1e-6, eps=0.01, adaptive_dt=False,
              dt_min=5e-4, dt_max=0.01, target_div=1e-4, Kp=0.5, Ki=0.05, Kd=0.1,
              flow_type="von_karman", advection_scheme="rk3", pressure_solver="multigrid",
              les_model="smagorinsky", limiter="minmod", v_cycles=1, fast_mode=False,
              brinkman_eta=0.005, grid_type="collocated", verbose=False, nn_pressure_model=None,
              *, mg_mode="parity", mg_rtol=1e-6, max_cycles=40, stream=None) -> SimState:
    """GB300 replacement of step_pure (solver/pure_functions/step.py:49-467).

    Same keywords and the same SimState result (torch CUDA tensors).  The LES
    field is not used on the collocated path, exactly as in the reference
    (:177-180).  ``advection_scheme='weno5'`` selects WENO5-JS advection;
    ``mg_mode='converge'`` replaces the fixed V-cycle count by the converging
    multigrid (relative residual ``mg_rtol``, warm-started from ``state.p``).
    Not on this path: the divergence-PID dt (``adaptive_dt=True``), and the CG,
    FFT and Jacobi solvers; asking for them raises."""
    if adaptive_dt:
        raise NotImplementedError("the divergence-PID time step is not part of the GB300 path")
    if pressure_solver not in ("multigrid", "nn"):
        raise NotImplementedError(f"pressure_solver={pressure_solver!r}: only multigrid runs on the GB300 path")
    if grid_type == "mac":
        # the reference's step_pure broadcasts (nx+1, ny) against (nx, ny) at
        # step.py:348 and fails for the MAC grid; use StepHandler(grid_type='mac')
        raise ValueError("step_pure does not support grid_type='mac' (it fails in the reference too)")
    u = _f32(state.u, "u")
    nx, ny = u.shape
    _f32(state.v, "v", (nx, ny))
    _f32(mask, "mask", (nx, ny))
    if sdf is not None:
        _f32(sdf, "sdf", (nx, ny))
    adv = "weno5" if advection_scheme == "weno5" else "upwind"
    warm = mg_mode == "converge" and state.p is not None
    cfg = StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=float(nu), U_inf=float(U_inf),
                     grid_type="collocated", flow_type=flow_type, variant="pure", use_les=False,
                     advection_scheme=adv, fast_mode=bool(fast_mode), brinkman_eta=float(brinkman_eta),
                     v_cycles=int(v_cycles), mg_mode=mg_mode, mg_rtol=mg_rtol, max_cycles=max_cycles,
                     warm_start=warm, has_sdf=sdf is not None, dt=float(state.dt))
    plan = get_plan(cfg, u.device)
    plan.prepare(mask, sdf, stream)
    p_guess = _f32(state.p, "p", (nx, ny)) if warm else None
    un, vn, p = run_step(plan, u, state.v, mask, p_guess, stream=stream, dt=float(state.dt))
    return SimState(u=un, v=vn, p=p, u_prev=state.u, v_prev=state.v, c=state.c, dt=state.dt,
                    iteration=state.iteration + 1, grid_type=state.grid_type,
                    integral=state.integral, prev_error=state.prev_error)


# ----------------------------------------------------------------- GUI step
class StepHandler:
    """BaselineSolver._step for one fixed configuration
    (solver/simulation/step_handlers.py:62-301).  Construct it with the values
    BaselineSolver holds (grid spacing, flow, sim_params, nu_hyper_ratio, sdf,
    slip_walls) and call ``_step(u, v, mask, dt)`` -> (u, v, p)."""

    def __init__(self, nx, ny, dx, dy, nu, U_inf=1.0, *, grid_type="collocated",
                 flow_type="von_karman", use_les=False, les_model="dynamic_smagorinsky",
                 smagorinsky_constant=0.17, nu_hyper_ratio=0.0, slip_walls=True, fast_mode=False,
                 brinkman_eta=1e-4, multigrid_v_cycles=5, sdf=None, dt=1e-3,
                 advection_scheme="upwind", mg_mode="parity", mg_rtol=1e-6, max_cycles=40,
                 cfl_dt=False, cfl_target=0.5, dt_min=1e-6, dt_max=1.0, warm_start=False):
        self.sdf = sdf
        self.dt = dt
        self.cfg = StepConfig(nx=nx, ny=ny, dx=dx, dy=dy, nu=nu, U_inf=U_inf, grid_type=grid_type,
                              flow_type=flow_type, variant="gui", use_les=use_les,
                              les_model=les_model, smagorinsky_constant=smagorinsky_constant,
                              advection_scheme=advection_scheme, fast_mode=fast_mode,
                              slip_walls=slip_walls, brinkman_eta=brinkman_eta,
                              nu_hyper_ratio=nu_hyper_ratio, v_cycles=multigrid_v_cycles,
                              mg_mode=mg_mode, mg_rtol=mg_rtol, max_cycles=max_cycles,
                              warm_start=warm_start, has_sdf=sdf is not None and grid_type == "collocated",
                              cfl_dt=cfl_dt, dt=dt, cfl_target=cfl_target, dt_min=dt_min,
                              dt_max=dt_max)
        self._plan = None

    def plan(self, device) -> Plan:
        if self._plan is None:
            self._plan = get_plan(self.cfg, device)
        return self._plan

    def _step(self, u, v, mask, dt=None, p_guess=None, out=None, stream=None):
        nx, ny = self.cfg.nx, self.cfg.ny
        mac = self.cfg.grid_type == "mac"
        _f32(u, "u", (nx + 1, ny) if mac else (nx, ny))
        _f32(v, "v", (nx, ny + 1) if mac else (nx, ny))
        _f32(mask, "mask", (nx, ny))
        plan = self.plan(u.device)
        plan.prepare(mask, self.sdf if self.cfg.has_sdf else None, stream)
        if warm_mode(self.cfg.warm_start) == 1 and p_guess is None:
            raise ValueError("warm_start needs p_guess")
        return run_step(plan, u, v, mask, p_guess if self.cfg.warm_start else None, out=out,
                        stream=stream, dt=dt if dt is not None else self.dt)

    def stats(self) -> dict:
        return self._plan.stats() if self._plan else {}


# ----------------------------------------------------------------- pressure
def _poisson(rhs, mask, dx, dy, levels, v_cycles, tolerance, flow_type, grid_type, mode="parity",
             rtol=1e-6, p0=None, max_cycles=40, stream=None, return_stats=False):
    _f32(rhs, "rhs")
    nx, ny = rhs.shape
    _f32(mask, "mask", (nx, ny))
    cfg = StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=1.0, grid_type=grid_type,
                     flow_type=flow_type, variant="gui", v_cycles=int(v_cycles), levels=int(levels),
                     mg_mode=mode, mg_rtol=rtol, mg_tolerance=float(tolerance),
                     max_cycles=max_cycles, warm_start=p0 is not None)
    plan = get_plan(cfg, rhs.device)
    plan.prepare(mask, None, stream)
    p = torch.empty_like(rhs)
    if p0 is not None:
        _f32(p0, "p0", (nx, ny))
    check("aj_poisson_mg", lib().aj_poisson_mg(ctypes.byref(plan.params), rhs.data_ptr(),
                                               mask.data_ptr(), _ptr(p0), p.data_ptr(),
                                               plan.ws.data_ptr(), plan.nbytes,
                                               plan.stats_buf.data_ptr(), _stream(stream)))
    if return_stats:
        return p, plan.stats()
    return p


def poisson_multigrid(rhs, mask, dx, dy, levels=4, v_cycles=5, tolerance=1e-6,
                      flow_type="von_karman", **kw):
    """pressure_solvers/multigrid_solver.py:55-241 on the GPU."""
    return _poisson(rhs, mask, dx, dy, levels, v_cycles, tolerance, flow_type, "collocated", **kw)


def poisson_multigrid_mac(rhs, mask, dx, dy, levels=4, v_cycles=5, tolerance=1e-6,
                          flow_type="von_karman", **kw):
    """pressure_solvers/multigrid_solver_mac.py:59-246 on the GPU."""
    return _poisson(rhs, mask, dx, dy, levels, v_cycles, tolerance, flow_type, "mac", **kw)


def poisson_multigrid_converge(rhs, mask, dx, dy, rtol=1e-6, p0=None, max_cycles=40, mac=False,
                               stream=None) -> Tuple[torch.Tensor, dict]:
    """Converging mode: solve the reference operator to ||b - A p|| <= rtol ||b||
    (FP64 refinement around FP32 red-black V-cycles).  Returns (p, stats)."""
    return _poisson(rhs, mask, dx, dy, 4, 1, 1e-6, "von_karman", "mac" if mac else "collocated",
                    mode="converge", rtol=rtol, p0=p0, max_cycles=max_cycles, stream=stream,
                    return_stats=True)


# ----------------------------------------------------------------- pieces
def constant_smagorinsky(u, v, dx, dy, delta, C_s=0.1, stream=None):
    """solver/les_models.py:179-200 (collocated inputs)."""
    _f32(u, "u")
    nx, ny = u.shape
    _f32(v, "v", (nx, ny))
    out = torch.empty_like(u)
    p = make_params(StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=1.0,
                               smagorinsky_constant=float(C_s), les_delta=float(delta),
                               mg_mode="none"))
    check("aj_les", lib().aj_les(ctypes.byref(p), 1, u.data_ptr(), v.data_ptr(), out.data_ptr(),
                                 None, None, 0, _stream(stream)))
    return out


def dynamic_smagorinsky(u, v, dx, dy, delta, alpha=2.0, stream=None):
    """solver/les_models.py:79-176 (collocated inputs); returns (nu_sgs, C_d)."""
    if alpha != 2.0:
        raise NotImplementedError("the test-filter ratio is fixed at alpha = 2 (les_models.py:80)")
    _f32(u, "u")
    nx, ny = u.shape
    _f32(v, "v", (nx, ny))
    cfg = StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=1.0, les_delta=float(delta),
                     mg_mode="none")
    plan = get_plan(cfg, u.device)
    out, cd = torch.empty_like(u), torch.empty_like(u)
    check("aj_les", lib().aj_les(ctypes.byref(plan.params), 2, u.data_ptr(), v.data_ptr(),
                                 out.data_ptr(), cd.data_ptr(), plan.ws.data_ptr(), plan.nbytes,
                                 _stream(stream)))
    return out, cd


def _predictor(grid_type, u, v, dt, nu, dx, dy, mask, sdf, U_inf, nu_sgs, nu_hyper_ratio,
               slip_walls, fast_mode, brinkman_eta, flow_type, double_count, advection, stream):
    nx, ny = mask.shape
    cfg = StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=float(nu), U_inf=float(U_inf),
                     grid_type=grid_type, flow_type=flow_type, variant="gui",
                     advection_scheme=advection, fast_mode=bool(fast_mode),
                     slip_walls=bool(slip_walls), brinkman_eta=float(brinkman_eta),
                     nu_hyper_ratio=float(nu_hyper_ratio), mg_mode="none",
                     has_sdf=sdf is not None, dt=float(dt))
    plan = get_plan(cfg, u.device)
    plan.prepare(mask, sdf, stream)
    us, vs = torch.empty_like(u), torch.empty_like(v)
    check("aj_predictor", lib().aj_predictor(ctypes.byref(plan.params), u.data_ptr(), v.data_ptr(),
                                             mask.data_ptr(), _ptr(nu_sgs), int(double_count),
                                             us.data_ptr(), vs.data_ptr(), plan.ws.data_ptr(),
                                             plan.nbytes, _stream(stream)))
    return us, vs


def rk_step_unified(u, v, dt, nu, dx, dy, mask, sdf=None, U_inf=1.0, nu_sgs=None,
                    nu_hyper_ratio=0.0, slip_walls=True, fast_mode=False, brinkman_eta=0.01,
                    flow_type="von_karman", *, double_count=False, advection="upwind",
                    stream=None):
    """advection_schemes/rk3_simple_new.py:175-358.  ``nu`` is the scalar
    viscosity; ``double_count=True`` reproduces the GUI call that passes
    nu + nu_sgs as nu together with nu_sgs (step_handlers.py:76,84-85)."""
    nx, ny = mask.shape
    _f32(u, "u", (nx, ny))
    _f32(v, "v", (nx, ny))
    return _predictor("collocated", u, v, dt, nu, dx, dy, mask, sdf, U_inf, nu_sgs, nu_hyper_ratio,
                      slip_walls, fast_mode, brinkman_eta, flow_type, double_count, advection,
                      stream)


def rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, U_inf=1.0, nu_sgs=None, nu_hyper_ratio=0.0,
                        slip_walls=True, fast_mode=False, brinkman_eta=0.01,
                        flow_type="von_karman", *, advection="upwind", stream=None):
    """advection_schemes/rk3_mac.py:220-504.  ``advection='weno5'`` replaces
    the reference's blended upwind and central advection terms by WENO5-JS
    derivatives on the faces."""
    nx, ny = mask.shape
    _f32(u, "u", (nx + 1, ny))
    _f32(v, "v", (nx, ny + 1))
    return _predictor("mac", u, v, dt, nu, dx, dy, mask, None, U_inf, nu_sgs, nu_hyper_ratio,
                      slip_walls, fast_mode, brinkman_eta, flow_type, False, advection, stream)


def compute_cfl_timestep(u, v, dx, dy, nu, mask=None, cfl_target=0.3, dt_min=1e-4, dt_max=0.01,
                         stream=None) -> torch.Tensor:
    """timestepping/cfl_adaptive_dt.py:6-71; returns a 1-element CUDA tensor."""
    mac = tuple(u.shape) != tuple(v.shape)
    nx = v.shape[0]
    ny = u.shape[1]
    p = make_params(StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=float(nu),
                               grid_type="mac" if mac else "collocated", cfl_target=cfl_target,
                               dt_min=dt_min, dt_max=dt_max, cfl_dt=True))
    scratch = torch.zeros(256, dtype=torch.uint8, device=u.device)
    out = torch.empty(1, dtype=torch.float32, device=u.device)
    check("aj_cfl_dt", lib().aj_cfl_dt(ctypes.byref(p), u.data_ptr(), v.data_ptr(), out.data_ptr(),
                                       scratch.data_ptr(), 256, _stream(stream)))
    return out


def diagnostics(u, v, dx, dy, grid_type="collocated", flow_type="von_karman", stream=None):
    """The post-step fields of step_for_visualization
    (solver/simulation/visualization_step.py:224-256): (vorticity, divergence,
    speed), each (nx, ny), computed on the device."""
    mac = grid_type == "mac"
    nx = v.shape[0]
    ny = u.shape[1]
    _f32(u, "u", (nx + 1, ny) if mac else (nx, ny))
    _f32(v, "v", (nx, ny + 1) if mac else (nx, ny))
    p = make_params(StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=1.0,
                               grid_type=grid_type, flow_type=flow_type))
    out = [torch.empty((nx, ny), dtype=torch.float32, device=u.device) for _ in range(3)]
    check("aj_diagnostics", lib().aj_diagnostics(ctypes.byref(p), u.data_ptr(), v.data_ptr(),
                                                 out[0].data_ptr(), out[1].data_ptr(),
                                                 out[2].data_ptr(), _stream(stream)))
    return tuple(out)


def post_step(u, v, c, dt, dx, dy, diffusivity, grid_type="collocated", flow_type="von_karman",
              diagnostics=True, stream=None):
    """The post-step epilogue in one kernel: the dye c advanced one step with
    the new velocity (scalar_advection_diffusion_*, solver/operators.py:111-150,
    solver/operators_mac.py:161-215; clipped to [0, 1]) and, with
    diagnostics, the fields of step_for_visualization.  Returns c_new, or
    (c_new, vorticity, divergence, speed)."""
    mac = grid_type == "mac"
    nx, ny = c.shape
    _f32(u, "u", (nx + 1, ny) if mac else (nx, ny))
    _f32(v, "v", (nx, ny + 1) if mac else (nx, ny))
    _f32(c, "c", (nx, ny))
    p = make_params(StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=1.0,
                               grid_type=grid_type, flow_type=flow_type))
    c_new = torch.empty_like(c)
    d = [torch.empty((nx, ny), dtype=torch.float32, device=u.device) for _ in range(3)] \
        if diagnostics else [None, None, None]
    ptr = lambda t: None if t is None else t.data_ptr()
    check("aj_post_step", lib().aj_post_step(ctypes.byref(p), u.data_ptr(), v.data_ptr(),
                                             c.data_ptr(), c_new.data_ptr(), float(dt),
                                             float(diffusivity), ptr(d[0]), ptr(d[1]), ptr(d[2]),
                                             _stream(stream)))
    return (c_new, *d) if diagnostics else c_new


def make_geometry(kind, nx, ny, lx, ly, geo, eps, device="cuda", stream=None):
    """Obstacle SDF and mask = 1 - sigmoid(-sdf/eps) on the device
    (solver/simulation/mask_generator.py:10-160).  kind: 'cylinder' (cx, cy, r),
    'naca4' (chord, aoa_deg, x_le, y_le, m, p, t), 'cyl3_row' / 'cyl3_tri'
    (cx, cy, diameter, spacing)."""
    mask = torch.empty((nx, ny), dtype=torch.float32, device=device)
    sdf = torch.empty((nx, ny), dtype=torch.float32, device=device)
    arr = (ctypes.c_double * 8)(*([float(g) for g in geo] + [0.0] * (8 - len(geo))))
    check("aj_geometry", lib().aj_geometry(nx, ny, float(lx), float(ly), _lib.GEOM[kind], arr,
                                           float(eps), mask.data_ptr(), sdf.data_ptr(),
                                           _stream(stream)))
    return mask, sdf
