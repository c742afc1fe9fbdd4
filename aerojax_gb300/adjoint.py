"""Gradients through step_pure rollouts on the GPU (reverse mode).

The reference differentiates its pure step with ``jax.grad``:
``differentiable_rollout`` scans step_pure (solver/solver.py:34-75) and
``design_loss`` / ``grad_design_loss`` differentiate a loss of the final
state with respect to the params dict (:78-114); the WIP optimizer does the
same through its own scan (inverse_design_WIP/optimizer_autodiff.py:113-205).
Here the forward rollout runs through aj_step and the reverse scan through
aj_step_vjp, one graph launch per step each; the cotangent of the final
state comes from the caller's loss.

Covered: the collocated von Karman step_pure with upwind RK3/RK2, a fixed dt
and the parity V-cycle (the configuration the reference's rollouts use), and
the collocated GUI step without LES (hyperviscosity and either wall
condition), the step the WIP optimizer differentiates.
Cotangents returned: the initial u, v; the SDF (through the Brinkman chi,
when one is given); nu and U_inf.
"""
from __future__ import annotations

import ctypes
from dataclasses import replace
from typing import Optional

import torch

from . import _lib
from ._lib import check, lib
from .params import SimState, StepConfig
from .solver import Plan, _f32, _ptr, _stream

__all__ = ["StepVjp", "step_pure_vjp", "gui_step_vjp", "differentiable_rollout", "rollout_vjp"]


def _config(nx, ny, dx, dy, nu, U_inf, dt, has_sdf, v_cycles=1, fast_mode=False,
            brinkman_eta=0.005) -> StepConfig:
    return StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=float(nu), U_inf=float(U_inf),
                      grid_type="collocated", flow_type="von_karman", variant="pure",
                      use_les=False, advection_scheme="upwind", fast_mode=bool(fast_mode),
                      brinkman_eta=float(brinkman_eta), v_cycles=int(v_cycles), mg_mode="parity",
                      warm_start=False, has_sdf=bool(has_sdf), dt=float(dt))


class StepVjp:
    """A prepared forward plan plus the reverse pass's workspace and fixed
    staging buffers (so that every call replays one cached graph)."""

    def __init__(self, cfg: StepConfig, device):
        self.cfg = cfg
        self.plan = Plan(cfg, device)
        nbytes = int(lib().aj_step_vjp_workspace_size(ctypes.byref(self.plan.params)))
        if nbytes == 0:
            raise ValueError("aj_step_vjp does not cover this configuration")
        self.adj_bytes = nbytes
        self.aws = torch.empty(nbytes, dtype=torch.uint8, device=device)
        shape = (cfg.nx, cfg.ny)
        z = lambda: torch.zeros(shape, dtype=torch.float32, device=device)
        self.u_in, self.v_in = z(), z()
        self.g_in = (z(), z(), z())          # cotangents of the step's u, v, p
        self.g_out = (z(), z())              # cotangents of the step's input u, v
        self.gsdf = z()
        self.gscal = torch.zeros(2, dtype=torch.float64, device=device)

    def prepare(self, mask, sdf=None, stream=None):
        self.plan.prepare(mask, sdf, stream)

    def kernel_count(self) -> int:
        return int(lib().aj_step_vjp_kernel_count(ctypes.byref(self.plan.params)))

    def __call__(self, u, v, mask, gu, gv, gp=None, stream=None):
        """Cotangents of one step's inputs, written to ``self.g_out``; the
        SDF's cotangent is added to ``self.gsdf`` and (d/d nu, d/d U_inf) to
        ``self.gscal``.  u, v, gu, gv, gp are copied into the staging buffers
        (skipped when they already are those buffers)."""
        for dst, src in ((self.u_in, u), (self.v_in, v), (self.g_in[0], gu), (self.g_in[1], gv)):
            if src.data_ptr() != dst.data_ptr():
                dst.copy_(src)
        gp_ptr = None
        if gp is not None:
            if gp.data_ptr() != self.g_in[2].data_ptr():
                self.g_in[2].copy_(gp)
            gp_ptr = self.g_in[2].data_ptr()
        P = self.plan
        check("aj_step_vjp", lib().aj_step_vjp(
            ctypes.byref(P.params), self.u_in.data_ptr(), self.v_in.data_ptr(), mask.data_ptr(),
            self.g_in[0].data_ptr(), self.g_in[1].data_ptr(), gp_ptr, self.g_out[0].data_ptr(),
            self.g_out[1].data_ptr(), self.gsdf.data_ptr() if self.cfg.has_sdf else None,
            self.gscal.data_ptr(), P.ws.data_ptr(), P.nbytes, self.aws.data_ptr(), self.adj_bytes,
            _stream(stream)))
        return self.g_out

    def zero_grad(self):
        self.gsdf.zero_()
        self.gscal.zero_()


def step_pure_vjp(state: SimState, mask, sdf, dx, dy, nu, U_inf, g_u, g_v, g_p=None, *,
                  v_cycles=1, fast_mode=False, brinkman_eta=0.005, stream=None) -> dict:
    """Reverse mode of one aerojax_gb300.step_pure call with the same
    arguments: returns the cotangents of state.u, state.v, the SDF (None
    without one), nu and U_inf from those of the new u, v and p."""
    u = _f32(state.u, "u")
    nx, ny = u.shape
    _f32(state.v, "v", (nx, ny))
    _f32(mask, "mask", (nx, ny))
    if sdf is not None:
        _f32(sdf, "sdf", (nx, ny))
    cfg = _config(nx, ny, dx, dy, nu, U_inf, state.dt, sdf is not None, v_cycles, fast_mode,
                  brinkman_eta)
    op = StepVjp(cfg, u.device)
    op.prepare(mask, sdf, stream)
    gu, gv = op(u, state.v, mask, g_u, g_v, g_p, stream=stream)
    sc = op.gscal.cpu()
    return {"u": gu.clone(), "v": gv.clone(), "sdf": op.gsdf.clone() if sdf is not None else None,
            "nu": float(sc[0]), "U_inf": float(sc[1])}


def gui_step_vjp(u, v, mask, dt, g_u, g_v, g_p=None, *, sdf=None, dx, dy, nu, U_inf=1.0,
                 nu_hyper_ratio=0.0, slip_walls=True, fast_mode=False, brinkman_eta=1e-4,
                 multigrid_v_cycles=5, stream=None) -> dict:
    """Reverse mode of the collocated GUI step without LES
    (BaselineSolver._step, step_handlers.py:62-185; the step the WIP
    optimizer scans under jax.grad, inverse_design_WIP/optimizer_autodiff.py
    :113-205), with StepHandler's keywords: the cotangents of u, v, the SDF
    (None without one), nu and U_inf from those of the new u, v and p."""
    u = _f32(u, "u")
    nx, ny = u.shape
    _f32(v, "v", (nx, ny))
    _f32(mask, "mask", (nx, ny))
    if sdf is not None:
        _f32(sdf, "sdf", (nx, ny))
    cfg = StepConfig(nx=nx, ny=ny, dx=float(dx), dy=float(dy), nu=float(nu), U_inf=float(U_inf),
                     grid_type="collocated", flow_type="von_karman", variant="gui",
                     use_les=False, advection_scheme="upwind", fast_mode=bool(fast_mode),
                     slip_walls=bool(slip_walls), brinkman_eta=float(brinkman_eta),
                     nu_hyper_ratio=float(nu_hyper_ratio), v_cycles=int(multigrid_v_cycles),
                     mg_mode="parity", warm_start=False, has_sdf=sdf is not None, dt=float(dt))
    op = StepVjp(cfg, u.device)
    op.prepare(mask, sdf, stream)
    gu, gv = op(u, v, mask, g_u, g_v, g_p, stream=stream)
    sc = op.gscal.cpu()
    return {"u": gu.clone(), "v": gv.clone(), "sdf": op.gsdf.clone() if sdf is not None else None,
            "nu": float(sc[0]), "U_inf": float(sc[1])}


def _rollout_config(state, params):
    if params.get("adaptive_dt", False):
        raise NotImplementedError("the divergence-PID time step is not differentiated on this path")
    if params.get("nn_pressure_model") is not None:
        raise NotImplementedError("nn_pressure_model is not differentiated on this path")
    sdf = params.get("sdf")
    u = _f32(state.u, "u")
    nx, ny = u.shape
    cfg = _config(nx, ny, params.get("dx", 0.01), params.get("dy", 0.01),
                  params.get("nu", 0.003), params.get("U_inf", 2.0), state.dt, sdf is not None)
    return cfg, sdf


# Plans, staging buffers and reverse-pass operators of the rollouts, kept per
# configuration: repeated rollouts replay the graphs captured by the first.
# Nothing in them carries over from one rollout to the next, so the oldest
# configuration is dropped beyond _MAX_CACHED.
_FWD: dict = {}
_REV: dict = {}
_MAX_CACHED = 8


def _cached(cache: dict, key, make):
    ent = cache.get(key)
    if ent is None:
        while len(cache) >= _MAX_CACHED:
            cache.pop(next(iter(cache)))
        ent = make()
        cache[key] = ent
    return ent


def _forward_plan(cfg: StepConfig, device):
    def make():
        shape = (cfg.nx, cfg.ny)
        e = lambda: torch.empty(shape, dtype=torch.float32, device=device)
        return (Plan(cfg, device), [(e(), e()), (e(), e())], e())
    ent = _cached(_FWD, (repr(replace(cfg, dt=0.0)), str(device)), make)
    ent[0].params.dt = float(cfg.dt)
    return ent


def _reverse_op(cfg: StepConfig, device) -> "StepVjp":
    op = _cached(_REV, (repr(replace(cfg, dt=0.0)), str(device)), lambda: StepVjp(cfg, device))
    op.plan.params.dt = float(cfg.dt)
    return op


def differentiable_rollout(initial_state: SimState, mask, params: dict, num_steps: int = 200,
                           stream=None):
    """solver/solver.py:34-75 on the GPU: ``num_steps`` step_pure calls with
    the params dict's values (same keys and defaults: dx, dy 0.01, nu 0.003,
    U_inf 2.0, sdf).  Returns (final_state, (u_hist, v_hist)), the history
    stacked like lax.scan's output, [num_steps, nx, ny] each."""
    cfg, sdf = _rollout_config(initial_state, params)
    dev = initial_state.u.device
    plan, bufs, p = _forward_plan(cfg, dev)
    plan.prepare(mask, sdf, stream)
    nx, ny = cfg.nx, cfg.ny
    hu = torch.empty((num_steps, nx, ny), dtype=torch.float32, device=dev)
    hv = torch.empty_like(hu)
    # fixed ping-pong buffers: one cached graph serves every step
    bufs[0][0].copy_(initial_state.u)
    bufs[0][1].copy_(initial_state.v)
    cur = 0
    for k in range(num_steps):
        (u, v), (uo, vo) = bufs[cur], bufs[1 - cur]
        check("aj_step", lib().aj_step(ctypes.byref(plan.params), u.data_ptr(), v.data_ptr(),
                                       mask.data_ptr(), None, uo.data_ptr(), vo.data_ptr(),
                                       p.data_ptr(), plan.ws.data_ptr(), plan.nbytes,
                                       plan.stats_buf.data_ptr(), _stream(stream)))
        hu[k].copy_(uo)
        hv[k].copy_(vo)
        cur = 1 - cur
    prev_u = hu[-2] if num_steps > 1 else initial_state.u
    prev_v = hv[-2] if num_steps > 1 else initial_state.v
    final = SimState(u=hu[-1], v=hv[-1], p=p.clone(), u_prev=prev_u, v_prev=prev_v,
                     c=initial_state.c,
                     dt=initial_state.dt, iteration=initial_state.iteration + num_steps,
                     grid_type="collocated", integral=initial_state.integral,
                     prev_error=initial_state.prev_error)
    return final, (hu, hv)


def rollout_vjp(initial_state: SimState, mask, params: dict, num_steps: int, g_u, g_v,
                history=None, stream=None) -> dict:
    """Reverse scan of differentiable_rollout: from the cotangent (g_u, g_v)
    of the final state's u, v, the cotangents of the initial u, v, of
    params['sdf'] (None without one), of params['nu'] and params['U_inf'].
    ``history`` is differentiable_rollout's second result (recomputed when
    absent)."""
    cfg, sdf = _rollout_config(initial_state, params)
    if history is None:
        _, history = differentiable_rollout(initial_state, mask, params, num_steps, stream)
    hu, hv = history
    op = _reverse_op(cfg, initial_state.u.device)
    op.prepare(mask, sdf, stream)
    op.zero_grad()
    gA = (op.g_in[0], op.g_in[1])
    gA[0].copy_(g_u)
    gA[1].copy_(g_v)
    for k in range(num_steps - 1, -1, -1):
        u_k = initial_state.u if k == 0 else hu[k - 1]
        v_k = initial_state.v if k == 0 else hv[k - 1]
        gu, gv = op(u_k, v_k, mask, gA[0], gA[1], None, stream=stream)
        gA[0].copy_(gu)
        gA[1].copy_(gv)
    sc = op.gscal.cpu()
    return {"u": gA[0].clone(), "v": gA[1].clone(),
            "sdf": op.gsdf.clone() if sdf is not None else None,
            "nu": float(sc[0]), "U_inf": float(sc[1])}
