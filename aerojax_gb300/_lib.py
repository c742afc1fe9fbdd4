"""ctypes binding of libaerojax_gb300.so (the C ABI in include/aerojax_gb300.h).

The library is the only compute path: if it is missing, importing the
functions that need it raises immediately; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
from ctypes import c_double, c_int32, c_size_t, c_void_p, POINTER

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libaerojax_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "aerojax_gb300.h")

# enums (include/aerojax_gb300.h)
AJ_OK, AJ_ERR_SHAPE, AJ_ERR_PARAM, AJ_ERR_NONFINITE, AJ_ERR_NOT_CONVERGED = 0, 1, 2, 3, 4
AJ_ERR_TIMEOUT, AJ_ERR_CUDA, AJ_ERR_WORKSPACE = 5, 6, 7
GRID = {"collocated": 0, "mac": 1}
FLOW = {"von_karman": 0, "lid_driven_cavity": 1, "taylor_green": 2}
VARIANT = {"pure": 0, "gui": 1}
LES = {None: 0, "none": 0, "smagorinsky": 1, "dynamic_smagorinsky": 2}
ADV = {"upwind": 0, "rk3": 0, "weno5": 1}
MG = {"parity": 0, "converge": 1, "none": 2}
GEOM = {"cylinder": 1, "naca4": 2, "cyl3_row": 3, "cyl3_tri": 4}

STATUS_NAMES = {0: "AJ_OK", 1: "AJ_ERR_SHAPE", 2: "AJ_ERR_PARAM", 3: "AJ_ERR_NONFINITE",
                4: "AJ_ERR_NOT_CONVERGED", 5: "AJ_ERR_TIMEOUT", 6: "AJ_ERR_CUDA",
                7: "AJ_ERR_WORKSPACE"}


class AjStepParams(ctypes.Structure):
    _fields_ = [(n, c_int32) for n in (
        "nx", "ny", "grid_type", "flow_type", "variant", "les_model", "advection", "mg_mode",
        "fast_mode", "slip_walls", "v_cycles", "levels", "max_cycles", "has_sdf", "cfl_dt",
        "warm_start", "nn_factor")] + [(n, c_double) for n in (
        "dx", "dy", "dt", "dt_correction", "nu", "U_inf", "brinkman_eta",
        "smagorinsky_constant", "nu_hyper_ratio", "mg_tolerance", "mg_rtol", "cfl_target",
        "dt_min", "dt_max", "les_delta")]


class AjStats(ctypes.Structure):
    _fields_ = [("cycles", c_int32), ("converged", c_int32), ("err", c_int32), ("pad", c_int32),
                ("rel_residual", c_double), ("rhs_norm", c_double), ("dt", c_double),
                ("abs_residual_sq", c_double)]


STATS_BYTES = ctypes.sizeof(AjStats)

_SIGS = {
    "aj_version": (c_int32, []),
    "aj_workspace_size": (c_size_t, [POINTER(AjStepParams)]),
    "aj_check_params": (c_int32, [POINTER(AjStepParams)]),
    "aj_prepare": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_size_t,
                             c_void_p]),
    "aj_step": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                          c_void_p, c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]),
    "aj_poisson_mg": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p, c_size_t, c_void_p, c_void_p]),
    "aj_les": (c_int32, [POINTER(AjStepParams), c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                         c_void_p, c_size_t, c_void_p]),
    "aj_predictor": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                               c_int32, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "aj_cfl_dt": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                            c_size_t, c_void_p]),
    "aj_geometry": (c_int32, [c_int32, c_int32, c_double, c_double, c_int32, POINTER(c_double),
                              c_double, c_void_p, c_void_p, c_void_p]),
    "aj_poisson_mg_static": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p]),
    "aj_kernel_count": (c_int32, [POINTER(AjStepParams), c_int32]),
    "aj_nn_param_count": (c_size_t, []),
    "aj_nn_packed_count": (c_size_t, []),
    "aj_nn_act_bytes": (c_size_t, [c_int32, c_int32, c_int32]),
    "aj_nn_input": (c_void_p, [c_int32, c_int32, c_int32, c_void_p]),
    "aj_nn_pack": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "aj_nn_forward": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_size_t,
                                c_void_p, c_void_p]),
    "aj_nn_backward": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_size_t, c_void_p, c_void_p]),
    "aj_nn_loss": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p]),
    "aj_nn_adam": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int32, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             c_void_p]),
    "aj_nn_expand": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "aj_nn_features": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "aj_workspace_rhs": (c_void_p, [POINTER(AjStepParams), c_void_p]),
    "aj_nn_warmstart": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "aj_step_nn": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_size_t, c_void_p, c_void_p]),
    "aj_profile_kernel": (c_int32, [POINTER(AjStepParams), c_int32, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_size_t, c_void_p]),
    "aj_release_graphs": (c_int32, []),
    "aj_diagnostics": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p, c_void_p]),
    "aj_step_host": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p, c_void_p, c_size_t, c_void_p, c_void_p]),
    "aj_post_step": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                               ctypes.c_float, ctypes.c_float, c_void_p, c_void_p, c_void_p,
                               c_void_p]),
    "aj_step_vjp_workspace_size": (c_size_t, [POINTER(AjStepParams)]),
    "aj_step_vjp": (c_int32, [POINTER(AjStepParams), c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_size_t, c_void_p, c_size_t, c_void_p]),
    "aj_step_vjp_kernel_count": (c_int32, [POINTER(AjStepParams)]),
    "aj_autotune": (c_int32, [POINTER(AjStepParams), c_void_p, c_size_t, c_int32,
                              POINTER(ctypes.c_float), POINTER(c_int32), c_void_p]),
    "aj_ffi_prepare": (c_void_p, [c_void_p]),
    "aj_ffi_step": (c_void_p, [c_void_p]),
    "aj_ensemble_step": (c_int32, [c_int32, POINTER(AjStepParams), POINTER(c_void_p),
                                   POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p),
                                   POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p),
                                   POINTER(c_void_p), POINTER(c_size_t), c_void_p, c_void_p]),
}

_lib = None


class AeroJaxError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, fn, status):
        self.status = status
        super().__init__(f"{fn} failed: {STATUS_NAMES.get(status, status)}")


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"aerojax_gb300 CUDA library not found at {LIB_PATH}; build it with "
                "`python -m aerojax_gb300.build` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(fn, status):
    if status != AJ_OK:
        if status == AJ_ERR_SHAPE:
            raise ValueError(f"{fn}: grid not suitable (AJ_ERR_SHAPE)")
        raise AeroJaxError(fn, status)


def header_symbols():
    """Names of every function the public header declares."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(
        r"^\s*(?:const\s+)?(?:int32_t|size_t|float|void)\s*\*?\s*(aj_\w+)\s*\(", text, re.M)))
