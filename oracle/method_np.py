"""The benchmark's method restated on the CPU — TEST INFRASTRUCTURE ONLY.

Used only by ``bench.py``'s CPU legs (its ``cpu_baseline`` and its
``--impl reference`` arm), never by the package.  It runs, with the oracle's
NumPy restatement of the reference (``ref_np``), the configuration the GPU
arm is measured on, so that the CPU number is for the same work:

  NACA 0012 on the MAC grid (chord 256 cells at 2048x512, leading edge at
  cell (400, 256), 10 deg), Re 1000, Smagorinsky C_s 0.17, the GUI step
  (solver/simulation/step_handlers.py:188-293) with dt from CFL 0.5
  (timestepping/cfl_adaptive_dt.py:6-71), the pressure solved to a 1e-6
  relative residual by the converging multigrid (ref_np.mg_converge), warm
  started from p1 + (dt/dt1)(p1 - p2) of the last two solutions, and, with
  the trained network, that guess corrected by the network's prediction
  (nn_np.features / forward / apply_correction, the GPU's data path).

The predictor runs in float32 (the reference's default precision,
solver/config.py:28); the multigrid and the network in float64.

``run_replicas`` runs independent replicas of the stepper, one process per
host core (multiprocessing 'spawn'), each timing its own steps after a
common start, and returns the aggregate cell-steps per second.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import nn_np as N
from . import ref_np as R


def naca_case(nx=2048, ny=512, seed=0):
    lx, ly = 32.0 * nx / 2048, 8.0 * ny / 512
    dx, dy = lx / nx, ly / ny
    X, Y = R.grid_coords(nx, ny, lx, ly)
    chord = 256 * dx * nx / 2048
    xle, yle = (400 * nx // 2048) * dx, (ny // 2) * dy
    sdf = R.sdf_naca4(X, Y, chord, 10.0, xle, yle, 0.0, 0.0, 0.12)
    f = np.float32
    mask = R.mask_from_sdf(sdf, 0.05 * dx).astype(f)
    rng = np.random.default_rng(seed)
    u = (1.0 + 1e-3 * rng.standard_normal((nx + 1, ny))).astype(f)
    v = np.zeros((nx, ny + 1), f)
    return dict(nx=nx, ny=ny, dx=dx, dy=dy, nu=chord / 1000.0, mask=mask, u=u, v=v)


class MethodStepper:
    """The GPU arm's step on the CPU.  mode: 'nn' (network-corrected
    extrapolation), 'extrap', 'plain' (zero guess), or 'reference' (the
    reference's own V-cycle, 5 cycles, the GUI default)."""

    def __init__(self, case, mode="nn", weights=None, factor=8, rtol=1e-6):
        self.c = case
        self.mode = mode
        self.F = factor
        self.rtol = rtol
        self.w = None
        if mode == "nn":
            with np.load(weights) as z:
                self.w = z["master"].astype(np.float64)
        self.hist = []          # (p, dt) of the last two solves
        self.cycles = []

    def _guess(self, b, dt):
        c = self.c
        if self.mode == "plain" or not self.hist:
            g = np.zeros_like(b)
        elif len(self.hist) == 1:
            g = self.hist[0][0].copy()
        else:
            (p1, dt1), (p2, _) = self.hist
            g = p1 + (dt / dt1) * (p1 - p2)
        if self.mode != "nn":
            return g
        x3, _, scale = N.features(b, c["mask"], g, c["dx"], c["dy"], self.F)
        h, w, _ = x3.shape
        x = np.zeros((h, w, N.IN_CH))
        x[..., :3] = x3
        y = N.forward(self.w, x)
        return N.apply_correction(y[..., 0], g, self.F, scale)

    def step(self, u, v):
        c = self.c
        f = np.float32
        dt = float(R.compute_cfl_timestep(u, v, c["dx"], c["dy"], c["nu"], 0.5, 1e-6, 1.0))
        kw = dict(sdf=None, dx=f(c["dx"]), dy=f(c["dy"]), nu=f(c["nu"]), U_inf=f(1.0),
                  grid_type="mac", use_les=True, les_model="smagorinsky",
                  smagorinsky_constant=f(0.17), brinkman_eta=f(1e-4))
        if self.mode == "reference":
            un, vn, p = R.step_gui(u, v, c["mask"], f(dt), v_cycles=5, **kw)
            return un, vn, p
        mg = R.MGConfig(mode="converge", rtol=self.rtol, max_cycles=60,
                        guess=lambda b: self._guess(b, dt))
        un, vn, p = R.step_gui(u, v, c["mask"], f(dt), mg=mg, **kw)
        self.cycles.append(mg.info.get("cycles", 0))
        self.hist = [(np.asarray(p, np.float64), dt)] + self.hist[:1]
        return un, vn, p


def _replica(k, nx, ny, mode, weights, steps, warmup, barrier, out, init):
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    case = naca_case(nx, ny, seed=k)
    st = MethodStepper(case, mode, weights)
    u, v = case["u"], case["v"]
    if init is not None:         # a developed state: velocities and the solve history
        with np.load(init) as z:
            u, v = z["u"].astype(np.float32), z["v"].astype(np.float32)
            st.hist = [(z["p1"].astype(np.float64), float(z["dt1"])),
                       (z["p2"].astype(np.float64), float(z["dt2"]))]
    for _ in range(warmup):
        u, v, _ = st.step(u, v)
    n0 = len(st.cycles)
    barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        u, v, _ = st.step(u, v)
    el = time.perf_counter() - t0
    cyc = st.cycles[n0:]
    out.put((k, el, float(np.mean(cyc)) if cyc else None))


def run_replicas(nx, ny, mode, weights, steps, warmup, procs=None, init=None):
    """Aggregate Mcell-steps/s of `procs` concurrent replicas (default: every
    core this process may run on), each from the seeded initial state or, with
    `init` (an .npz of u, v, p1, dt1, p2, dt2), from that developed state.
    Returns (value, info)."""
    import multiprocessing as mp
    if procs is None:
        procs = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(procs)
    out = ctx.Queue()
    saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS",
                                             "MKL_NUM_THREADS")}
    for v in saved:
        os.environ[v] = "1"          # one thread per replica, inherited at spawn
    try:
        ps = [ctx.Process(target=_replica, args=(k, nx, ny, mode, weights, steps, warmup,
                                                 barrier, out, init)) for k in range(procs)]
        for p in ps:
            p.start()
        res = [out.get() for _ in ps]
        for p in ps:
            p.join()
    finally:
        for v, val in saved.items():
            if val is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = val
    el = max(r[1] for r in res)
    value = procs * nx * ny * steps / el / 1e6
    cyc = [r[2] for r in res if r[2] is not None]
    return value, {"procs": procs, "seconds": el, "per_replica_s_per_step": el / steps,
                   "mg_cycles_mean": float(np.mean(cyc)) if cyc else None}
