"""Host-side parameter logic mirrored from the reference (no device work).

SimState mirrors solver/params.py:11-31; grid coordinates follow
solver/params.py:33-61 (dx = lx/nx while the coordinates are
linspace(0, lx, nx)); the Reynolds-number presets follow
solver/params.py:233-254 and 308-413.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional


@dataclass
class SimState:
    """Simulation state (solver/params.py:11-31) holding torch CUDA tensors.

    Collocated: u, v, p are (nx, ny).  MAC: u (nx+1, ny), v (nx, ny+1),
    p (nx, ny)."""
    u: Any
    v: Any
    p: Any
    u_prev: Any
    v_prev: Any
    c: Any
    dt: float
    iteration: int
    grid_type: str = "collocated"
    integral: float = 0.0
    prev_error: float = 0.0


@dataclass
class GridParams:
    """solver/params.py:33-61 (coordinates are produced on demand)."""
    nx: int
    ny: int
    lx: float
    ly: float

    @property
    def dx(self) -> float:
        return self.lx / self.nx

    @property
    def dy(self) -> float:
        return self.ly / self.ny

    def x(self, i: float) -> float:
        """Physical x of cell index i: linspace(0, lx, nx)[i]."""
        return i * self.lx / (self.nx - 1)

    def y(self, j: float) -> float:
        return j * self.ly / (self.ny - 1)


def compute_eps_multiplier(Re: float) -> float:
    """solver/params.py:233-254."""
    if Re <= 2000:
        return 0.05
    if Re <= 5000:
        return 0.03
    return 0.02


def get_re_parameters(Re: float, grid_nx: int = 512) -> dict:
    """Re-dependent stability presets, solver/params.py:308-413."""
    p = {"C_s": 0.1, "nu_hyper_ratio": 0.0, "advection_scheme": "rk3_simple", "nu_h": 0.0,
         "brinkman_eta": 1e-4, "dt_max": 0.01, "cfl_target": 0.3, "use_les": True}
    rows = [
        (1e3, dict(C_s=0.08, nu_hyper_ratio=0.0, advection_scheme="rk3_simple", nu_h=0.0,
                   brinkman_eta=1e-4, dt_max=0.005, cfl_target=0.3)),
        (1e4, dict(C_s=0.1, nu_hyper_ratio=0.01, advection_scheme="rk3_simple", nu_h=0.0,
                   brinkman_eta=1e-4, dt_max=0.008, cfl_target=0.25)),
        (1e5, dict(C_s=0.12, nu_hyper_ratio=0.03, advection_scheme="rk3_simple", nu_h=0.0,
                   brinkman_eta=1e-6, dt_max=0.008, cfl_target=0.35)),
        (1e6, dict(C_s=0.15, nu_hyper_ratio=0.05, advection_scheme="rk3_high", nu_h=1e-5,
                   brinkman_eta=1e-7, dt_max=0.006, cfl_target=0.3)),
        (1e7, dict(C_s=0.18, nu_hyper_ratio=0.08, advection_scheme="rk3_high", nu_h=2e-5,
                   brinkman_eta=1e-7, dt_max=0.004, cfl_target=0.25)),
    ]
    for lim, upd in rows:
        if Re <= lim:
            p.update(upd)
            break
    else:
        p.update(C_s=0.20, nu_hyper_ratio=0.1, advection_scheme="rk3_high", nu_h=3e-5,
                 brinkman_eta=1e-7, dt_max=0.003, cfl_target=0.2)
    if grid_nx < 512:
        p["C_s"] *= 1.2
        p["nu_hyper_ratio"] *= 1.5
        p["brinkman_eta"] *= 1.2
        p["cfl_target"] *= 0.8
    return p


@dataclass
class StepConfig:
    """Every option of one projection step, in the reference's vocabulary.

    variant 'pure' is step_pure (solver/pure_functions/step.py:49-467);
    variant 'gui' is BaselineSolver._step (step_handlers.py:62-301)."""
    nx: int
    ny: int
    dx: float
    dy: float
    nu: float
    U_inf: float = 1.0
    grid_type: str = "collocated"
    flow_type: str = "von_karman"
    variant: str = "pure"
    use_les: bool = False
    les_model: str = "smagorinsky"
    smagorinsky_constant: float = 0.1
    advection_scheme: str = "upwind"
    fast_mode: bool = False
    slip_walls: bool = True
    brinkman_eta: float = 0.005
    nu_hyper_ratio: float = 0.0
    v_cycles: int = 1
    levels: int = 4
    mg_mode: str = "parity"
    mg_rtol: float = 1e-6
    mg_tolerance: float = 1e-6
    max_cycles: int = 40
    warm_start: Any = False       # False/True (p_guess) or "extrapolate"
    nn_factor: int = 0
    has_sdf: bool = False
    cfl_dt: bool = False
    dt: float = 1e-3
    dt_correction: float = 0.0
    cfl_target: float = 0.5
    dt_min: float = 1e-6
    dt_max: float = 1.0
    les_delta: float = 0.0
    nn_model: Optional[Any] = None
