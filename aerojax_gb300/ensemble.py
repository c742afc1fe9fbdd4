"""Batched ensemble: many independent cylinder-channel simulations of uneven
grid sizes stepped together as one CUDA graph launch (aj_ensemble_step).

The reference steps one simulation at a time; the ensemble workload here is
64 instances with sizes drawn from {256x64, 512x96, 768x192, 1024x256},
cylinder diameter uniform in 8-32 cells, centre at 10-20 % of nx and 40-60 %
of ny, Re log-uniform in [100, 1000]; float32, RK3 with WENO5-JS advection,
converging multigrid to a 1e-6 relative residual.  Each instance is the
collocated step_pure step (solver/pure_functions/step.py:49-467) of the
cylinder channel (grid spacing 1/64, inlet U = 1, slip walls), the flow of
solver/params.py:308-413's presets at its Re.  The level-0 multigrid tile
shape of every grid size comes from the autotuner (aj_autotune).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from ._lib import AjStats, AjStepParams, check, lib
from .params import StepConfig, compute_eps_multiplier, get_re_parameters
from .solver import Plan, _stream, make_geometry

SIZES = [(256, 64), (512, 96), (768, 192), (1024, 256)]
H = 1.0 / 64.0          # grid spacing of every instance


@dataclass
class Instance:
    nx: int
    ny: int
    d_cells: float
    cx_frac: float
    cy_frac: float
    re: float


def draw_instances(n=64, seed=0, sizes=SIZES) -> List[Instance]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, ny = sizes[int(rng.integers(len(sizes)))]
        out.append(Instance(nx, ny, float(rng.uniform(8, 32)), float(rng.uniform(0.1, 0.2)),
                            float(rng.uniform(0.4, 0.6)),
                            float(math.exp(rng.uniform(math.log(100.0), math.log(1000.0))))))
    return out


def instance_case(spec: Instance, device, seed=0, warm_start="extrapolate", advection="weno5",
                  rtol=1e-6):
    """StepConfig, mask, sdf and the seeded initial state of one instance."""
    nx, ny = spec.nx, spec.ny
    lx, ly = nx * H, ny * H
    D = spec.d_cells * H
    U = 1.0
    nu = U * D / spec.re
    eps = compute_eps_multiplier(spec.re) * H
    cx, cy = spec.cx_frac * lx, spec.cy_frac * ly
    mask, sdf = make_geometry("cylinder", nx, ny, lx, ly, (cx, cy, D / 2), eps, device)
    re = get_re_parameters(spec.re, nx)
    cfg = StepConfig(nx=nx, ny=ny, dx=H, dy=H, nu=nu, U_inf=U, grid_type="collocated",
                     variant="pure", advection_scheme=advection, brinkman_eta=re["brinkman_eta"],
                     mg_mode="converge", mg_rtol=rtol, max_cycles=60, warm_start=warm_start,
                     has_sdf=True, cfl_dt=True, dt=0.5 * H, cfl_target=0.5, dt_min=1e-6,
                     dt_max=1.0)
    rng = np.random.default_rng(seed)
    u = torch.as_tensor((1.0 + 1e-3 * rng.standard_normal((nx, ny))).astype(np.float32),
                        device=device)
    v = torch.zeros((nx, ny), dtype=torch.float32, device=device)
    return cfg, mask, sdf, u, v


def _ptrs(ts):
    return (ctypes.c_void_p * len(ts))(*[None if t is None else t.data_ptr() for t in ts])


class Ensemble:
    """n instances, each with its own workspace and two state buffers; step()
    advances all of them with one graph launch."""

    def __init__(self, specs: List[Instance], device="cuda", seed=0, warm_start="extrapolate",
                 advection="weno5", rtol=1e-6, tune=True):
        self.device = torch.device(device)
        self.specs = specs
        self.n = len(specs)
        self.plans, self.masks, self.bufs = [], [], []
        for k, spec in enumerate(specs):
            cfg, mask, sdf, u, v = instance_case(spec, self.device, seed + k, warm_start,
                                                 advection, rtol)
            plan = Plan(cfg, self.device)
            plan.prepare(mask, sdf)
            self.plans.append(plan)
            self.masks.append((mask, sdf))
            p = torch.zeros_like(u)
            self.bufs.append([(u, v, p), (torch.empty_like(u), torch.empty_like(v),
                                          torch.empty_like(u))])
        self.tuned = {}
        if tune:
            for plan in self.plans:
                key = (plan.cfg.nx, plan.cfg.ny)
                if key not in self.tuned:
                    self.tuned[key] = autotune(plan)
        self.params = (AjStepParams * self.n)(*[pl.params for pl in self.plans])
        self.ws = _ptrs([pl.ws for pl in self.plans])
        self.ws_bytes = (ctypes.c_size_t * self.n)(*[pl.nbytes for pl in self.plans])
        self.mask_ptrs = _ptrs([m for m, _ in self.masks])
        self.stats_buf = torch.zeros(self.n * _lib.STATS_BYTES, dtype=torch.uint8,
                                     device=self.device)
        self.cur = 0
        self._arrays = {}
        for c in (0, 1):
            src = [b[c] for b in self.bufs]
            dst = [b[1 - c] for b in self.bufs]
            self._arrays[c] = tuple(_ptrs(x) for x in (
                [s[0] for s in src], [s[1] for s in src], [s[2] for s in src],
                [d[0] for d in dst], [d[1] for d in dst], [d[2] for d in dst]))

    @property
    def cells(self) -> int:
        return sum(s.nx * s.ny for s in self.specs)

    def state(self, k):
        """(u, v, p) of instance k after the last step."""
        return self.bufs[k][self.cur]

    def step(self, stream=None):
        u, v, p, uo, vo, po = self._arrays[self.cur]
        check("aj_ensemble_step", lib().aj_ensemble_step(
            self.n, self.params, u, v, self.mask_ptrs, p, uo, vo, po, self.ws, self.ws_bytes,
            self.stats_buf.data_ptr(), _stream(stream)))
        self.cur = 1 - self.cur

    def stats(self) -> List[dict]:
        raw = bytes(self.stats_buf.cpu().numpy().tobytes())
        out = []
        for k in range(self.n):
            s = AjStats.from_buffer_copy(raw[k * _lib.STATS_BYTES:(k + 1) * _lib.STATS_BYTES])
            out.append({"cycles": s.cycles, "converged": bool(s.converged), "err": s.err,
                        "rel_residual": s.rel_residual, "dt": s.dt})
        return out


def autotune(plan: Plan, reps: int = 10, stream=None) -> dict:
    """Runs aj_autotune for the plan's grid shape; returns the per-candidate
    times (ms) and the chosen level-0 tile variant."""
    times = (ctypes.c_float * 3)()
    chosen = ctypes.c_int32(0)
    check("aj_autotune", lib().aj_autotune(ctypes.byref(plan.params), plan.ws.data_ptr(),
                                           plan.nbytes, reps, times, ctypes.byref(chosen),
                                           _stream(stream)))
    return {"times_ms": list(times), "chosen": int(chosen.value)}
