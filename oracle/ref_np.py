"""CPU oracle for the AeroJAX projection step — TEST INFRASTRUCTURE ONLY.

This module checks the product and is never part of it.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and its
``--impl reference`` arm) may import it.  The shipped package
``aerojax_gb300`` never imports it and has no CPU fallback.

What it is: a NumPy restatement of the reference's hot path, evaluated in
float64 by default (``dtype=np.float32`` reproduces the reference's default
FP32 arithmetic order closely enough to serve as the timed CPU baseline).
Every function cites the reference lines it follows (paths are relative to the
AeroJAX project root).  ``jnp.pad``/``jnp.roll`` map to ``np.pad``/``np.roll``
with the same modes; ``x.at[idx].set(y)`` maps to a copy plus an assignment.

Parity pinning: the reference ships no tests and no golden vectors.  JAX is
not installed here, so the fixtures in ``tests/golden/`` are produced by
executing the reference's *own source files* under a small NumPy stand-in for
the jax API (``tests/golden/jax_numpy_shim.py``) in float64, and this
restatement is checked against them.  XLA's own float32 rounding is therefore
not pinned; the float64 results of the reference's algorithm are.

Deliberate, documented reference behaviours reproduced here:
  * the RK3 stages restart from ``u`` (not the stage value) before the
    Brinkman division (``advection_schemes/rk3_simple_new.py:315-337``);
  * multigrid coarse levels reuse the fine dx, dy; prolongation leaves the last
    fine row and column zero; the smoother is undamped Jacobi
    (``pressure_solvers/multigrid_solver.py:134-217``);
  * the GUI collocated step double-counts the eddy viscosity
    (``solver/simulation/step_handlers.py:76,84-85``);
  * LES gradients are periodic (``solver/les_models.py:43-46`` via
    ``solver/operators.py:11-38``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

FLOW_TYPES = ("von_karman", "lid_driven_cavity", "taylor_green")


# ---------------------------------------------------------------------------
# small helpers
# ---------------------------------------------------------------------------
def _f(x, dtype):
    return np.asarray(x, dtype=dtype)


def sigmoid(x):
    """jax.nn.sigmoid: logistic function, evaluated stably."""
    x = np.asarray(x)
    out = np.empty_like(x)
    pos = x >= 0
    out[pos] = 1.0 / (1.0 + np.exp(-x[pos]))
    ex = np.exp(x[~pos])
    out[~pos] = ex / (1.0 + ex)
    return out


# ---------------------------------------------------------------------------
# finite-difference operators — solver/operators.py, solver/operators_mac.py
# ---------------------------------------------------------------------------
def grad_x(f, dx):
    """solver/operators.py:11-14 (periodic)."""
    return (np.roll(f, -1, axis=0) - np.roll(f, 1, axis=0)) / (2.0 * dx)


def grad_y(f, dy):
    """solver/operators.py:35-38 (periodic)."""
    return (np.roll(f, -1, axis=1) - np.roll(f, 1, axis=1)) / (2.0 * dy)


def grad_x_nonperiodic(f, dx):
    """solver/operators.py:17-32: central interior, one-sided at the edges."""
    g = np.zeros_like(f)
    g[1:-1, :] = (f[2:, :] - f[:-2, :]) / (2.0 * dx)
    g[0, :] = (f[1, :] - f[0, :]) / dx
    g[-1, :] = (f[-1, :] - f[-2, :]) / dx
    return g


def grad_y_nonperiodic(f, dy):
    """solver/operators.py:41-56."""
    g = np.zeros_like(f)
    g[:, 1:-1] = (f[:, 2:] - f[:, :-2]) / (2.0 * dy)
    g[:, 0] = (f[:, 1] - f[:, 0]) / dy
    g[:, -1] = (f[:, -1] - f[:, -2]) / dy
    return g


def divergence(u, v, dx, dy):
    """solver/operators.py:75-78 (periodic)."""
    return grad_x(u, dx) + grad_y(v, dy)


def divergence_nonperiodic(u, v, dx, dy):
    """solver/operators.py:81-96: interior only, boundary ring = 0."""
    d = np.zeros_like(u)
    d[1:-1, 1:-1] = ((u[2:, 1:-1] - u[:-2, 1:-1]) / (2.0 * dx)
                     + (v[1:-1, 2:] - v[1:-1, :-2]) / (2.0 * dy))
    return d


def vorticity_nonperiodic(u, v, dx, dy):
    """solver/operators.py:105-108."""
    return grad_x_nonperiodic(v, dx) - grad_y_nonperiodic(u, dy)


def grad_x_staggered(f, dx):
    """solver/operators_mac.py:15-25 and 40-46 (identical bodies)."""
    fp = np.pad(f, ((1, 1), (0, 0)), mode="edge")
    return (fp[1:, :] - fp[:-1, :]) / dx


def grad_y_staggered(f, dy):
    """solver/operators_mac.py:28-37 and 49-55."""
    fp = np.pad(f, ((0, 0), (1, 1)), mode="edge")
    return (fp[:, 1:] - fp[:, :-1]) / dy


def divergence_staggered(u, v, dx, dy):
    """solver/operators_mac.py:58-80 (periodic and non-periodic are the same)."""
    return (u[1:, :] - u[:-1, :]) / dx + (v[:, 1:] - v[:, :-1]) / dy


def interpolate_to_cell_center(u, v):
    """solver/operators_mac.py:118-127."""
    return 0.5 * (u[1:, :] + u[:-1, :]), 0.5 * (v[:, 1:] + v[:, :-1])


def vorticity(u, v, dx, dy):
    """solver/operators.py:99-102 (periodic)."""
    return grad_x(v, dx) - grad_y(u, dy)


def vorticity_staggered(u, v, dx, dy):
    """solver/operators_mac.py:83-98, as written: d(u_centre)/dx - d(v_centre)/dy
    with periodic central differences (the names say dv/dx and du/dy, the
    arrays are the other velocity component)."""
    uc, vc = interpolate_to_cell_center(u, v)
    return ((np.roll(uc, -1, axis=0) - np.roll(uc, 1, axis=0)) / (2.0 * dx)
            - (np.roll(vc, -1, axis=1) - np.roll(vc, 1, axis=1)) / (2.0 * dy))


def vorticity_nonperiodic_staggered(u, v, dx, dy):
    """solver/operators_mac.py:101-115, the same pairing with edge padding."""
    uc, vc = interpolate_to_cell_center(u, v)
    up = np.pad(uc, ((1, 1), (0, 0)), mode="edge")
    vp = np.pad(vc, ((0, 0), (1, 1)), mode="edge")
    return (up[2:, :] - up[:-2, :]) / (2.0 * dx) - (vp[:, 2:] - vp[:, :-2]) / (2.0 * dy)


def diagnostics(u, v, dx, dy, mac=False, periodic=False):
    """Post-step fields of step_for_visualization
    (solver/simulation/visualization_step.py:224-256): vorticity, divergence
    and the speed |u| of the cell-centred velocity."""
    if mac:
        vort = (vorticity_staggered if periodic else vorticity_nonperiodic_staggered)(u, v, dx, dy)
        div = divergence_staggered(u, v, dx, dy)
        uc, vc = interpolate_to_cell_center(u, v)
    else:
        vort = (vorticity if periodic else vorticity_nonperiodic)(u, v, dx, dy)
        div = (divergence if periodic else divergence_nonperiodic)(u, v, dx, dy)
        uc, vc = u, v
    return vort, div, np.sqrt(uc * uc + vc * vc)


def scalar_advection_diffusion(c, u, v, dt, dx, dy, kappa, mac=False, periodic=False):
    """One explicit step of the passive scalar (dye): c + dt (-(u, v).grad c +
    kappa lap c), clipped to [0, 1].  The four variants of the reference:
      collocated, periodic      solver/operators.py:111-129 (the Laplacian
                                divides all five points by dx^2)
      collocated, non-periodic  solver/operators.py:132-150 (one-sided d/dx at
                                the inlet and outlet rows, periodic d/dy;
                                Laplacian edge-padded in x, periodic in y)
      MAC, periodic             solver/operators_mac.py:161-187 (face-averaged
                                velocities, periodic central differences,
                                edge-padded Laplacian)
      MAC, non-periodic         solver/operators_mac.py:189-215 (central
                                differences and Laplacian edge-padded)"""
    c = np.asarray(c)
    if mac:
        uc, vc = interpolate_to_cell_center(u, v)
        if periodic:
            dcx = (np.roll(c, -1, 0) - np.roll(c, 1, 0)) / (2.0 * dx)
            dcy = (np.roll(c, -1, 1) - np.roll(c, 1, 1)) / (2.0 * dy)
        else:
            px = np.pad(c, ((1, 1), (0, 0)), mode="edge")
            py = np.pad(c, ((0, 0), (1, 1)), mode="edge")
            dcx = (px[2:, :] - px[:-2, :]) / (2.0 * dx)
            dcy = (py[:, 2:] - py[:, :-2]) / (2.0 * dy)
        pe = np.pad(c, ((1, 1), (1, 1)), mode="edge")
        lap = ((pe[2:, 1:-1] + pe[:-2, 1:-1] - 2 * c) / dx ** 2
               + (pe[1:-1, 2:] + pe[1:-1, :-2] - 2 * c) / dy ** 2)
        adv = uc * dcx + vc * dcy
    elif periodic:
        dcx = (np.roll(c, -1, 0) - np.roll(c, 1, 0)) / (2.0 * dx)
        dcy = (np.roll(c, -1, 1) - np.roll(c, 1, 1)) / (2.0 * dy)
        lap = (np.roll(c, 1, 0) + np.roll(c, -1, 0) + np.roll(c, 1, 1) + np.roll(c, -1, 1)
               - 4 * c) / dx ** 2
        adv = u * dcx + v * dcy
    else:
        dcx = grad_x_nonperiodic(c, dx)
        dcy = (np.roll(c, -1, 1) - np.roll(c, 1, 1)) / (2.0 * dy)
        px = np.pad(c, ((1, 1), (0, 0)), mode="edge")
        lap = ((px[2:, :] - 2 * c + px[:-2, :]) / (dx * dx)
               + (np.roll(c, 1, 1) + np.roll(c, -1, 1) - 2 * c) / (dy * dy))
        adv = u * dcx + v * dcy
    return np.clip(c + dt * (-adv + kappa * lap), 0.0, 1.0)


def interpolate_to_x_face(c):
    """solver/operators_mac.py:130-137."""
    cp = np.pad(c, ((1, 1), (0, 0)), mode="edge")
    return 0.5 * (cp[1:, :] + cp[:-1, :])


def interpolate_to_y_face(c):
    """solver/operators_mac.py:140-147."""
    cp = np.pad(c, ((0, 0), (1, 1)), mode="edge")
    return 0.5 * (cp[:, 1:] + cp[:, :-1])


# ---------------------------------------------------------------------------
# LES — solver/les_models.py
# ---------------------------------------------------------------------------
def strain_rate(u, v, dx, dy):
    """solver/les_models.py:22-54 (collocated branch; periodic gradients)."""
    du_dx, du_dy = grad_x(u, dx), grad_y(u, dy)
    dv_dx, dv_dy = grad_x(v, dx), grad_y(v, dy)
    sxx, syy, sxy = du_dx, dv_dy, 0.5 * (du_dy + dv_dx)
    smag = np.sqrt(2.0 * (sxx ** 2 + syy ** 2 + 2.0 * sxy ** 2) + 1e-10)
    return smag, (du_dx, du_dy, dv_dx, dv_dy)


def box_filter_2d(f, filter_ratio=2):
    """solver/les_models.py:57-76: (2r+1)^2 periodic box average."""
    acc = np.zeros_like(f)
    for i in range(-filter_ratio, filter_ratio + 1):
        for j in range(-filter_ratio, filter_ratio + 1):
            acc = acc + np.roll(np.roll(f, i, axis=0), j, axis=1)
    return acc / ((2 * filter_ratio + 1) ** 2)


def constant_smagorinsky(u, v, dx, dy, delta, C_s=0.1):
    """solver/les_models.py:179-200 (collocated inputs)."""
    smag, _ = strain_rate(u, v, dx, dy)
    return (C_s * delta) ** 2 * smag


def dynamic_smagorinsky(u, v, dx, dy, delta, alpha=2.0):
    """solver/les_models.py:79-176: Germano-Lilly with a 5x5 periodic test
    filter, 3x3 interior average of LM and MM, C_d clipped to [0, 0.2]."""
    smag, (du_dx, du_dy, dv_dx, dv_dy) = strain_rate(u, v, dx, dy)
    ut, vt = box_filter_2d(u), box_filter_2d(v)
    smag_t, _ = strain_rate(ut, vt, dx, dy)
    uut, uvt, vvt = box_filter_2d(u * u), box_filter_2d(u * v), box_filter_2d(v * v)
    L11, L12, L22 = ut * ut - uut, ut * vt - uvt, vt * vt - vvt
    sxx_t = grad_x(ut, dx)
    syy_t = grad_y(vt, dy)
    sxy_t = 0.5 * (grad_y(ut, dy) + grad_x(vt, dx))
    sxx, syy, sxy = du_dx, dv_dy, 0.5 * (du_dy + dv_dx)
    ssxx = box_filter_2d(smag * sxx)
    ssxy = box_filter_2d(smag * sxy)
    ssyy = box_filter_2d(smag * syy)
    a2 = alpha ** 2
    M11 = a2 * smag_t * sxx_t - ssxx
    M12 = a2 * smag_t * sxy_t - ssxy
    M22 = a2 * smag_t * syy_t - ssyy

    def local_average(f):
        out = np.zeros_like(f)
        out[1:-1, 1:-1] = (f[1:-1, 1:-1] + f[2:, 1:-1] + f[:-2, 1:-1]
                           + f[1:-1, 2:] + f[1:-1, :-2] + f[2:, 2:] + f[2:, :-2]
                           + f[:-2, 2:] + f[:-2, :-2]) / 9.0
        return out

    LM = local_average(L11 * M11 + L12 * M12 + L22 * M22)
    MM = local_average(M11 * M11 + M12 * M12 + M22 * M22)
    Cd = np.clip(LM / (MM + 1e-8), 0.0, 0.2)
    return Cd * (delta * delta) * smag, Cd


# ---------------------------------------------------------------------------
# boundary conditions
# ---------------------------------------------------------------------------
def bc_collocated(u, v, U_inf, flow_type="von_karman", slip_walls=True):
    """advection_schemes/rk3_simple_new.py:250-280 (in place on copies)."""
    u, v = u.copy(), v.copy()
    if flow_type == "lid_driven_cavity":
        u[:, -1] = U_inf
        u[:, 0] = 0.0
        u[0, :] = 0.0
        u[-1, :] = 0.0
        v[:, 0] = 0.0
        v[:, -1] = 0.0
        v[0, :] = 0.0
        v[-1, :] = 0.0
    elif flow_type == "taylor_green":
        pass
    else:
        u[0, :] = U_inf
        v[0, :] = 0.0
        u[-1, :] = u[-2, :]
        v[-1, :] = v[-2, :]
        if slip_walls:
            u[:, 0] = u[:, 1]
            u[:, -1] = u[:, -2]
        else:
            u[:, 0] = 0.0
            u[:, -1] = 0.0
        v[:, 0] = 0.0
        v[:, -1] = 0.0
    return u, v


def bc_mac(u, v, U_inf, flow_type="von_karman", slip_walls=True):
    """advection_schemes/rk3_mac.py:292-330."""
    u, v = u.copy(), v.copy()
    if flow_type == "lid_driven_cavity":
        u[:, -1] = U_inf
        u[:, 0] = 0.0
        u[0, :] = 0.0
        u[-1, :] = 0.0
        v[:, 0] = 0.0
        v[:, -1] = 0.0
        v[0, :] = 0.0
        v[-1, :] = 0.0
    elif flow_type == "taylor_green":
        pass
    else:
        u[0, :] = U_inf
        v[0, :] = 0.0
        u[-1, :] = u[-2, :]
        v[-1, :] = v[-2, :]
        if slip_walls:
            u[:, 0] = u[:, 1]
            u[:, -1] = u[:, -2]
        else:
            u[:, 0] = 0.0
            u[:, -1] = 0.0
        v[:, 0] = 0.0
        v[:, -1] = 0.0
    return u, v


# ---------------------------------------------------------------------------
# RK3 / RK2 predictor — advection_schemes/rk3_simple_new.py:175-358
# ---------------------------------------------------------------------------
def rk_step_unified(u, v, dt, nu, dx, dy, mask, sdf=None, U_inf=1.0, nu_sgs=None,
                    nu_hyper_ratio=0.0, slip_walls=True, fast_mode=False,
                    brinkman_eta=0.01, flow_type="von_karman", advection="upwind"):
    """Collocated predictor.  ``nu`` may be a scalar or a field (the GUI step
    passes nu + nu_sgs here, step_handlers.py:76,84).  ``advection='weno5'``
    selects the WENO5-JS flux (a new option; see :func:`weno5_advection`)."""
    if sdf is not None:
        chi = sigmoid(-sdf / (0.1 * dx))                       # :194-198
    else:
        chi = 1.0 - mask                                       # :199-200
    eta = brinkman_eta
    pad_mode = "wrap" if flow_type == "taylor_green" else "edge"   # :205

    def laplacian(f):                                          # :215-219
        fp = np.pad(f, ((1, 1), (1, 1)), mode=pad_mode)
        return ((fp[2:, 1:-1] + fp[:-2, 1:-1] - 2 * f) / dx ** 2
                + (fp[1:-1, 2:] + fp[1:-1, :-2] - 2 * f) / dy ** 2)

    def upwind_advection(fld, vu, vv):                         # :287-298
        fpx = np.pad(fld, ((1, 1), (0, 0)), mode=pad_mode)
        fx = np.where(vu > 0, vu * (fld - fpx[:-2, :]) / dx, vu * (fpx[2:, :] - fld) / dx)
        fpy = np.pad(fld, ((0, 0), (1, 1)), mode=pad_mode)
        fy = np.where(vv > 0, vv * (fld - fpy[:, :-2]) / dy, vv * (fpy[:, 2:] - fld) / dy)
        return fx + fy

    def rhs_explicit(ui, vi):                                  # :284-313
        if advection == "weno5":
            adv_u = weno5_advection(ui, ui, vi, dx, dy, pad_mode)
            adv_v = weno5_advection(vi, ui, vi, dx, dy, pad_mode)
        else:
            adv_u = upwind_advection(ui, ui, vi)
            adv_v = upwind_advection(vi, ui, vi)
        lap_u, lap_v = laplacian(ui), laplacian(vi)
        nu_total = nu if nu_sgs is None else nu + nu_sgs
        ru = -adv_u + nu_total * lap_u
        rv = -adv_v + nu_total * lap_v
        if nu_hyper_ratio > 0:
            nu_h = nu * nu_hyper_ratio * (dx * dy)             # sponge disabled (=1), :282
            ru = ru - nu_h * laplacian(lap_u)
            rv = rv - nu_h * laplacian(lap_v)
        return ru, rv

    den = 1 + dt * chi / eta
    if not fast_mode:                                          # :315-337
        k1u, k1v = rhs_explicit(u, v)
        u2, v2 = (u + dt * k1u) / den, (v + dt * k1v) / den
        k2u, k2v = rhs_explicit(u2, v2)
        us, vs = u + dt * k2u, v + dt * k2v
        u3, v3 = (0.75 * u + 0.25 * us) / den, (0.75 * v + 0.25 * vs) / den
        k3u, k3v = rhs_explicit(u3, v3)
        us, vs = u + dt * k3u, v + dt * k3v
        un = ((1 / 3) * u + (2 / 3) * us) / den
        vn = ((1 / 3) * v + (2 / 3) * vs) / den
    else:                                                      # :339-353
        k1u, k1v = rhs_explicit(u, v)
        us, vs = (u + dt * k1u) / den, (v + dt * k1v) / den
        k2u, k2v = rhs_explicit(us, vs)
        un = (u + 0.5 * dt * (k1u + k2u)) / den
        vn = (v + 0.5 * dt * (k1v + k2v)) / den
    un = np.where(mask > 0.5, un, 0.0)
    vn = np.where(mask > 0.5, vn, 0.0)
    return bc_collocated(un, vn, U_inf, flow_type, slip_walls)


# ---------------------------------------------------------------------------
# WENO5-JS advection (new option; the reference plumbs weno_epsilon but never
# uses it: solver/pure_functions/step.py:52).  Restates Jiang & Shu (1996),
# "Efficient implementation of weighted ENO schemes", J. Comput. Phys. 126:
# fifth-order upwind-biased reconstruction of the derivative f_x with linear
# weights (1/10, 6/10, 3/10), smoothness indicators beta_k and eps=1e-6,
# applied in advective (non-conservative) form  vel * f_x, upwinded on the
# sign of vel exactly like the reference's first-order scheme.
# ---------------------------------------------------------------------------
WENO_EPS = 1e-6


def _weno5_minus(v1, v2, v3, v4, v5, eps=WENO_EPS):
    """Left-biased reconstruction at i+1/2 from differences v1..v5 =
    d_{i-2..i+2}; returns the WENO5-JS value."""
    b1 = 13.0 / 12.0 * (v1 - 2 * v2 + v3) ** 2 + 0.25 * (v1 - 4 * v2 + 3 * v3) ** 2
    b2 = 13.0 / 12.0 * (v2 - 2 * v3 + v4) ** 2 + 0.25 * (v2 - v4) ** 2
    b3 = 13.0 / 12.0 * (v3 - 2 * v4 + v5) ** 2 + 0.25 * (3 * v3 - 4 * v4 + v5) ** 2
    a1 = 0.1 / (eps + b1) ** 2
    a2 = 0.6 / (eps + b2) ** 2
    a3 = 0.3 / (eps + b3) ** 2
    s = a1 + a2 + a3
    q1 = v1 / 3.0 - 7.0 / 6.0 * v2 + 11.0 / 6.0 * v3
    q2 = -v2 / 6.0 + 5.0 / 6.0 * v3 + v4 / 3.0
    q3 = v3 / 3.0 + 5.0 / 6.0 * v4 - v5 / 6.0
    return (a1 * q1 + a2 * q2 + a3 * q3) / s


def weno5_derivative(f, vel, h, axis, pad_mode):
    """Upwind WENO5 approximation of df/dx_axis at every point.

    With d_k = (f_{k+1} - f_k)/h (one-sided differences), the left-biased
    derivative (vel > 0) is the WENO5 combination of d_{i-3..i+1} and the
    right-biased one (vel <= 0) the mirrored combination of d_{i+2..i-2}
    (Jiang & Shu 1996, Sec. 2, Hamilton-Jacobi form).  Ghost values follow the
    reference's padding mode (edge or wrap), three cells deep."""
    pw = [(0, 0), (0, 0)]
    pw[axis] = (3, 3)
    fp = np.pad(f, pw, mode=pad_mode)
    d = np.diff(fp, axis=axis) / h          # length n+5; d[k] = (fp[k+1]-fp[k])/h
    n = f.shape[axis]

    def sl(k):
        idx = [slice(None), slice(None)]
        idx[axis] = slice(k, k + n)
        return d[tuple(idx)]
    # point i (in padded coords i+3): backward differences d[i+3-1-m]
    dm = _weno5_minus(sl(0), sl(1), sl(2), sl(3), sl(4))      # d_{i-3}..d_{i+1}
    dp = _weno5_minus(sl(5), sl(4), sl(3), sl(2), sl(1))      # d_{i+2}..d_{i-2}
    return np.where(vel > 0, dm, dp)


def weno5_advection(fld, vu, vv, dx, dy, pad_mode):
    return (vu * weno5_derivative(fld, vu, dx, 0, pad_mode)
            + vv * weno5_derivative(fld, vv, dy, 1, pad_mode))


# ---------------------------------------------------------------------------
# MAC predictor — advection_schemes/rk3_mac.py:220-504
# ---------------------------------------------------------------------------
def v_to_u_face(vf):
    """v (nx, ny+1) at the u faces (nx+1, ny): rk3_mac.py:239-245."""
    vc = 0.5 * (vf[:, 1:] + vf[:, :-1])
    vp = np.pad(vc, ((1, 1), (0, 0)), mode="edge")
    return 0.5 * (vp[1:, :] + vp[:-1, :])


def u_to_v_face(uf):
    """u (nx+1, ny) at the v faces (nx, ny+1): rk3_mac.py:247-253."""
    uc = 0.5 * (uf[1:, :] + uf[:-1, :])
    up = np.pad(uc, ((0, 0), (1, 1)), mode="edge")
    return 0.5 * (up[:, 1:] + up[:, :-1])


def mac_advection_terms(uw, vw, dx, dy, nonper=True, scheme="upwind"):
    """(u.grad) u on the u faces and (u.grad) v on the v faces from the
    boundary-conditioned working copies uw (nx+1, ny), vw (nx, ny+1), before
    the face-mask factor.

    scheme='upwind' is the reference (rk3_mac.py:373-417): along the face
    normal a tanh blend alpha = (1 + tanh(u/0.05))/2 of the backward and
    forward differences (edge or wrap padding), across it a central
    difference (one-sided at the walls, or periodic) times the interpolated
    velocity.

    scheme='weno5' (new; the reference has no WENO5) uses the upwind WENO5-JS
    derivative of :func:`weno5_derivative` for both directions of both
    components, upwinded on the sign of the advecting velocity at the face,
    with ghost values three cells deep by edge (non-periodic) or wrap
    padding: adv_u = uw d_x^W(uw) + v_at_u d_y^W(uw), adv_v = u_at_v
    d_x^W(vw) + vw d_y^W(vw)."""
    v_at_u, u_at_v = v_to_u_face(vw), u_to_v_face(uw)
    pm = "edge" if nonper else "wrap"
    if scheme == "weno5":
        adv_u = (uw * weno5_derivative(uw, uw, dx, 0, pm)
                 + v_at_u * weno5_derivative(uw, v_at_u, dy, 1, pm))
        adv_v = (u_at_v * weno5_derivative(vw, u_at_v, dx, 0, pm)
                 + vw * weno5_derivative(vw, vw, dy, 1, pm))
        return adv_u, adv_v
    upx = np.pad(uw, ((1, 1), (0, 0)), mode=pm)
    back = (uw - upx[:-2, :]) / dx
    fwd = (upx[2:, :] - uw) / dx
    al = 0.5 * (1 + np.tanh(uw / 0.05))
    adv_ux = uw * (al * back + (1 - al) * fwd)
    if nonper:
        du_dy = np.zeros_like(uw)
        du_dy[:, 1:-1] = (uw[:, 2:] - uw[:, :-2]) / (2.0 * dy)
        du_dy[:, 0] = (uw[:, 1] - uw[:, 0]) / dy
        du_dy[:, -1] = (uw[:, -1] - uw[:, -2]) / dy
    else:
        du_dy = (np.roll(uw, -1, axis=1) - np.roll(uw, 1, axis=1)) / (2.0 * dy)
    adv_u = adv_ux + v_at_u * du_dy
    vpy = np.pad(vw, ((0, 0), (1, 1)), mode=pm)
    back = (vw - vpy[:, :-2]) / dy
    fwd = (vpy[:, 2:] - vw) / dy
    al = 0.5 * (1 + np.tanh(vw / 0.05))
    adv_vy = vw * (al * back + (1 - al) * fwd)
    if nonper:
        dv_dx = np.zeros_like(vw)
        dv_dx[1:-1, :] = (vw[2:, :] - vw[:-2, :]) / (2.0 * dx)
        dv_dx[0, :] = (vw[1, :] - vw[0, :]) / dx
        dv_dx[-1, :] = (vw[-1, :] - vw[-2, :]) / dx
    else:
        dv_dx = (np.roll(vw, -1, axis=0) - np.roll(vw, 1, axis=0)) / (2.0 * dx)
    adv_v = u_at_v * dv_dx + adv_vy
    return adv_u, adv_v


def rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, U_inf=1.0, nu_sgs=None,
                        nu_hyper_ratio=0.0, slip_walls=True, fast_mode=False,
                        brinkman_eta=0.01, flow_type="von_karman", advection="upwind"):
    """Staggered predictor.  ``advection='weno5'`` replaces the blended
    upwind and central terms by WENO5-JS derivatives (a new option; see
    :func:`mac_advection_terms`)."""
    chi = 1.0 - mask                                           # :231
    eta_safe = max(brinkman_eta, 1e-10)                        # :234
    nonper = flow_type in ("von_karman", "lid_driven_cavity")

    def lap_face(f, axis):                                     # :268-290
        if slip_walls:
            fp = np.pad(f, ((1, 1), (1, 1)), mode="symmetric")
        elif axis == 0:
            fy = np.pad(f, ((0, 0), (1, 1)), mode="constant")
            fy[:, 0] = -f[:, 0]
            fy[:, -1] = -f[:, -1]
            fp = np.pad(fy, ((1, 1), (0, 0)), mode="edge")
        else:
            fx = np.pad(f, ((1, 1), (0, 0)), mode="constant")
            fx[0, :] = -f[0, :]
            fx[-1, :] = -f[-1, :]
            fp = np.pad(fx, ((0, 0), (1, 1)), mode="edge")
        return ((fp[2:, 1:-1] + fp[:-2, 1:-1] - 2 * f) / dx ** 2
                + (fp[1:-1, 2:] + fp[1:-1, :-2] - 2 * f) / dy ** 2)

    mask_u = interpolate_to_x_face(mask)
    mask_v = interpolate_to_y_face(mask)

    def adv_terms(ui, vi):                                     # :332-417
        uw, vw = bc_mac(ui, vi, U_inf, flow_type, slip_walls)  # working copies, :381
        adv_u, adv_v = mac_advection_terms(uw, vw, dx, dy, nonper, advection)
        return adv_u * mask_u, adv_v * mask_v

    def rhs_explicit(ui, vi):                                  # :425-458
        au, av = adv_terms(ui, vi)
        lu, lv = lap_face(ui, 0), lap_face(vi, 1)
        if nu_sgs is None:
            ntu = ntv = nu
        else:
            ntu = nu + interpolate_to_x_face(nu_sgs)
            ntv = nu + interpolate_to_y_face(nu_sgs)
        ru = -au + ntu * lu
        rv = -av + ntv * lv
        if nu_hyper_ratio > 0:
            nh = nu * nu_hyper_ratio * (dx * dy)
            ru = ru - nh * lap_face(lu, 0)
            rv = rv - nh * lap_face(lv, 1)
        return ru, rv

    chi_u = interpolate_to_x_face(chi)                          # :462-463
    chi_v = interpolate_to_y_face(chi)
    du_ = 1 + dt * chi_u / eta_safe
    dv_ = 1 + dt * chi_v / eta_safe
    if not fast_mode:                                          # :465-486
        k1u, k1v = rhs_explicit(u, v)
        u2, v2 = (u + dt * k1u) / du_, (v + dt * k1v) / dv_
        k2u, k2v = rhs_explicit(u2, v2)
        us, vs = u + dt * k2u, v + dt * k2v
        u3, v3 = (0.75 * u + 0.25 * us) / du_, (0.75 * v + 0.25 * vs) / dv_
        k3u, k3v = rhs_explicit(u3, v3)
        us, vs = u + dt * k3u, v + dt * k3v
        un = ((1 / 3) * u + (2 / 3) * us) / du_
        vn = ((1 / 3) * v + (2 / 3) * vs) / dv_
    else:                                                      # :488-501
        k1u, k1v = rhs_explicit(u, v)
        us, vs = (u + dt * k1u) / du_, (v + dt * k1v) / dv_
        k2u, k2v = rhs_explicit(us, vs)
        un = (u + 0.5 * dt * (k1u + k2u)) / du_
        vn = (v + 0.5 * dt * (k1v + k2v)) / dv_
    un = np.where(chi_u < 0.5, un, 0.0)
    vn = np.where(chi_v < 0.5, vn, 0.0)
    return bc_mac(un, vn, U_inf, flow_type, slip_walls)


# ---------------------------------------------------------------------------
# multigrid, parity mode — pressure_solvers/multigrid_solver.py:55-241 and
# pressure_solvers/multigrid_solver_mac.py:59-246
# ---------------------------------------------------------------------------
def mg_levels_ok(nx, ny, levels=4):
    """Level count logic of multigrid_solver.py:96-106.  Returns max_levels,
    or raises ValueError exactly where the reference would fail (including the
    shape mismatch its prolongation would hit on non-divisible grids)."""
    max_levels, tx, ty = 1, nx, ny
    while tx % 2 == 0 and ty % 2 == 0 and max_levels < levels:
        tx //= 2
        ty //= 2
        max_levels += 1
    if max_levels < 2:
        raise ValueError(f"Grid dimensions ({nx}, {ny}) not suitable for multigrid "
                         f"with {levels} levels. Grid must be divisible by 2^{levels}")
    # the recursion restricts max_levels times; each prolongation must recover
    # the fine shape, and restrict() degenerates below 2 cells (:115-116)
    n, m = nx, ny
    for _ in range(max_levels):
        if n % 2 or m % 2 or n // 2 < 2 or m // 2 < 2:
            raise ValueError(f"Grid dimensions ({nx}, {ny}) not suitable for multigrid "
                             f"with {levels} levels (coarse shape mismatch)")
        n, m = n // 2, m // 2
    return max_levels


def _restrict(f):
    """multigrid_solver.py:108-132: unscaled 2x2 average."""
    n, m = f.shape[0] // 2, f.shape[1] // 2
    fe = f[:2 * n, :2 * m]
    return 0.25 * (fe[::2, ::2] + fe[1::2, ::2] + fe[::2, 1::2] + fe[1::2, 1::2])


def _prolong(c):
    """multigrid_solver.py:134-156: inject to even indices; interior odd
    indices interpolated; last fine row and column stay zero."""
    n, m = c.shape
    f = np.zeros((2 * n, 2 * m), dtype=c.dtype)
    f[::2, ::2] = c
    if 2 * n > 2:
        f[1:-1:2, ::2] = 0.5 * (f[0:-2:2, ::2] + f[2::2, ::2])
    if 2 * m > 2:
        f[::2, 1:-1:2] = 0.5 * (f[::2, 0:-2:2] + f[::2, 2::2])
    if 2 * n > 2 and 2 * m > 2:
        f[1:-1:2, 1:-1:2] = 0.25 * (f[0:-2:2, 0:-2:2] + f[2::2, 0:-2:2]
                                    + f[0:-2:2, 2::2] + f[2::2, 2::2])
    return f


def poisson_multigrid(rhs, mask, dx, dy, levels=4, v_cycles=5, tolerance=1e-6,
                      flow_type="von_karman", mac=False, p0=None, return_info=False):
    """Parity-mode V-cycle.  ``mac=False`` follows multigrid_solver.py:55-241,
    ``mac=True`` follows multigrid_solver_mac.py:59-246 (b *= mask, smoother
    multiplies by the level mask, Laplacian outlet row zeroed).  ``p0`` is an
    optional initial guess (the reference always starts from zero, :219)."""
    nx, ny = rhs.shape
    dt_ = rhs.dtype
    b = rhs * mask if mac else rhs.copy()
    if flow_type == "von_karman":
        b = b.copy()
        b[-1, :] = 0.0
    elif flow_type == "lid_driven_cavity":
        b = b - np.mean(b)
    max_levels = mg_levels_ok(nx, ny, levels)
    ax = 1.0 / (dx * dx)
    ay = 1.0 / (dy * dy)
    pm = "edge" if flow_type in ("von_karman", "lid_driven_cavity") else "wrap"

    def smooth(p, bl, ml, nu):
        for _ in range(nu):
            pp = np.pad(p, ((1, 1), (1, 1)), mode="edge")
            p = (ax * (pp[2:, 1:-1] + pp[:-2, 1:-1]) + ay * (pp[1:-1, 2:] + pp[1:-1, :-2]) - bl) \
                / (2.0 * (ax + ay))
            if mac:
                p = p * ml
        return p

    def apply_lap(p):
        pp = np.pad(p, ((1, 1), (1, 1)), mode=pm)
        lap = ax * (pp[2:, 1:-1] + pp[:-2, 1:-1] - 2 * p) + ay * (pp[1:-1, 2:] + pp[1:-1, :-2] - 2 * p)
        if mac and flow_type == "von_karman":
            lap[-1, :] = 0.0
        return lap

    def v_cycle(p, bl, ml, level):
        if level >= max_levels:
            return smooth(p, bl, ml, 10)
        p = smooth(p, bl, ml, 2)
        if flow_type == "von_karman":
            p = p.copy()
            p[-1, :] = 0.0
        r = bl - apply_lap(p)
        rc = _restrict(r)
        mc = (_restrict(ml) > 0.5).astype(dt_)
        ec = v_cycle(np.zeros_like(rc), rc, mc, level + 1)
        p = p + _prolong(ec)
        p = smooth(p, bl, ml, 2)
        if flow_type == "von_karman":
            p = p.copy()
            p[-1, :] = 0.0
        return p

    p = np.zeros((nx, ny), dtype=dt_) if p0 is None else np.array(p0, dtype=dt_)
    converged = False
    cycles = 0
    for _ in range(v_cycles):
        if not converged:
            p = v_cycle(p, b, mask, 0)
            cycles += 1
        r = b - apply_lap(p)
        converged = bool(np.sum(r ** 2) * dx * dy < tolerance ** 2)
    if flow_type == "lid_driven_cavity":
        p = p - p[nx // 2, ny // 2]
    if return_info:
        return p, {"cycles": cycles, "converged": converged}
    return p


def poisson_multigrid_mac(rhs, mask, dx, dy, levels=4, v_cycles=5, tolerance=1e-6,
                          flow_type="von_karman", p0=None):
    """pressure_solvers/multigrid_solver_mac.py:59-246."""
    return poisson_multigrid(rhs, mask, dx, dy, levels, v_cycles, tolerance, flow_type,
                             mac=True, p0=p0)


# ---------------------------------------------------------------------------
# corner smoothing — solver/pure_functions/corner_smoothing.py:39-61
# ---------------------------------------------------------------------------
def corner_smooth_pressure_gradient(dp_dx, ny, width=10):
    dp_dx = dp_dx.copy()
    idx = np.arange(width)
    fac = np.sin(np.pi / 2 * (idx / width)) ** 2
    dp_dx[0, idx] = dp_dx[0, idx] * fac
    top = ny - 1 - np.arange(width)
    dp_dx[0, top] = dp_dx[0, top] * fac
    return dp_dx


# ---------------------------------------------------------------------------
# time step — timestepping/cfl_adaptive_dt.py:6-71
# ---------------------------------------------------------------------------
def compute_cfl_timestep(u, v, dx, dy, nu, cfl_target=0.3, dt_min=1e-4, dt_max=0.01):
    EPS = 1e-12
    h = min(dx, dy)
    if u.shape != v.shape:
        maxv = max(np.max(np.abs(u)), np.max(np.abs(v)))
    else:
        maxv = np.max(np.sqrt(u ** 2 + v ** 2))
    dt = min(h / (maxv + EPS), 0.25 * h * h / (nu + EPS)) * cfl_target
    return float(max(dt_min, min(dt_max, dt)))


# ---------------------------------------------------------------------------
# the pressure-solve dispatch shared by both step variants
# ---------------------------------------------------------------------------
@dataclass
class MGConfig:
    """Which solver finishes the pressure equation.

    mode='parity'   : the reference's V-cycle, ``v_cycles`` cycles, zero guess.
    mode='converge' : converging multigrid to ``rtol`` relative residual with
                      an optional warm start ``p0``, or ``guess(b)`` computed
                      from the solve's right-hand side (see :func:`mg_converge`).
    """
    mode: str = "parity"
    v_cycles: int = 3
    levels: int = 4
    rtol: float = 1e-6
    max_cycles: int = 40
    p0: object = None
    guess: object = None        # callable b -> p0 (converging mode), overrides p0
    info: dict = field(default_factory=dict)


def _solve_pressure(rhs, mask, dx, dy, mg: MGConfig, flow_type, mac):
    if mg.mode == "parity":
        return poisson_multigrid(rhs, mask, dx, dy, mg.levels, mg.v_cycles, 1e-6,
                                 flow_type, mac=mac)
    b = rhs * mask if mac else rhs
    p0 = mg.guess(b) if mg.guess is not None else mg.p0
    p, info = mg_converge(b, dx, dy, rtol=mg.rtol, max_cycles=mg.max_cycles, p0=p0)
    mg.info.update(info)
    return p.astype(rhs.dtype)


# ---------------------------------------------------------------------------
# step_pure — solver/pure_functions/step.py:49-467 (collocated; the MAC branch
# of step_pure broadcasts (nx+1,ny) against (nx,ny) at :348 and cannot run)
# ---------------------------------------------------------------------------
def step_pure(u, v, dt, mask, sdf, dx, dy, nu, U_inf, use_les=False, smagorinsky_constant=0.1,
              les_model="smagorinsky", v_cycles=1, fast_mode=False, brinkman_eta=0.005,
              flow_type="von_karman", mg: MGConfig | None = None, advection="upwind"):
    """Returns (u_new, v_new, p).  The LES field is computed but not passed to
    the predictor on the collocated path (:177-180), so use_les changes nothing
    here; nu_hyper_ratio is hard-wired to 0 (:178)."""
    if mg is None:
        mg = MGConfig(mode="parity", v_cycles=v_cycles)
    us, vs = rk_step_unified(u, v, dt, nu, dx, dy, mask, sdf=sdf, U_inf=U_inf, nu_sgs=None,
                             nu_hyper_ratio=0.0, slip_walls=True, fast_mode=fast_mode,
                             brinkman_eta=brinkman_eta, flow_type=flow_type, advection=advection)
    if flow_type == "von_karman":                              # :182-191
        us, vs = us.copy(), vs.copy()
        us[0, :] = U_inf
        vs[0, :] = 0.0
        us[:, 0] = us[:, 1]
        us[:, -1] = us[:, -2]
        vs[:, 0] = 0.0
        vs[:, -1] = 0.0
    if flow_type in ("von_karman", "lid_driven_cavity"):
        div = divergence_nonperiodic(us, vs, dx, dy)
    else:
        div = divergence(us, vs, dx, dy)
    rhs = (div * mask) / dt                                    # :199
    p = _solve_pressure(rhs, mask, dx, dy, mg, flow_type, mac=False)
    if flow_type == "von_karman":                              # :259-264
        dpx, dpy = grad_x_nonperiodic(p, dx), grad_y_nonperiodic(p, dy)
        dmx, dmy = grad_x_nonperiodic(mask, dx), grad_y_nonperiodic(mask, dy)
    else:
        dpx, dpy = grad_x(p, dx), grad_y(p, dy)
        dmx, dmy = grad_x(mask, dx), grad_y(mask, dy)
    gm = np.sqrt(dmx ** 2 + dmy ** 2)                          # :313-335
    iface = gm > 0.1 / dx
    nxv = dmx / (gm + 1e-8)
    nyv = dmy / (gm + 1e-8)
    dn = dpx * nxv + dpy * nyv
    dpx = np.where(iface, dpx - dn * nxv, dpx)
    dpy = np.where(iface, dpy - dn * nyv, dpy)
    if flow_type == "von_karman":
        dpx = dpx.copy()
        dpx[0, :] = 0.0                                        # :341
    un = us - dt * dpx
    vn = vs - dt * dpy
    un = np.where(mask > 0.5, un, 0.0)
    vn = np.where(mask > 0.5, vn, 0.0)
    if flow_type == "von_karman":                              # :365-377
        un[0, :] = U_inf
        vn[0, :] = 0.0
        un[-1, :] = un[-2, :]
        vn[-1, :] = vn[-2, :]
        un[:, 0] = un[:, 1]
        un[:, -1] = un[:, -2]
        vn[:, 0] = 0.0
        vn[:, -1] = 0.0
    elif flow_type == "lid_driven_cavity":                     # :378-390
        un[:, -1] = 1.0
        un[:, 0] = 0.0
        un[0, :] = 0.0
        un[-1, :] = 0.0
        vn[:, 0] = 0.0
        vn[:, -1] = 0.0
        vn[0, :] = 0.0
        vn[-1, :] = 0.0
    un = np.where(mask > 0.5, un, 0.0)                         # :396-397
    vn = np.where(mask > 0.5, vn, 0.0)
    return un, vn, p


# ---------------------------------------------------------------------------
# GUI step — solver/simulation/step_handlers.py:62-293
# ---------------------------------------------------------------------------
def step_gui(u, v, mask, dt, *, sdf, dx, dy, nu, U_inf, grid_type="collocated", use_les=False,
             les_model="smagorinsky", smagorinsky_constant=0.17, nu_hyper_ratio=0.0,
             slip_walls=True, fast_mode=False, brinkman_eta=1e-4, flow_type="von_karman",
             v_cycles=5, dt_correction=None, mg: MGConfig | None = None, advection="upwind",
             return_nu_sgs=False):
    """BaselineSolver._step (step_handlers.py:296-301).  ``dt_correction`` is
    the trace-time ``self.dt`` used by the correction (:139, :252); it equals
    ``dt`` in the GUI.  Startup ramp is disabled (initializers.py:29)."""
    if mg is None:
        mg = MGConfig(mode="parity", v_cycles=v_cycles)
    if dt_correction is None:
        dt_correction = dt
    delta = (dx * dy) ** 0.5
    nu_sgs = None
    if grid_type == "mac":
        if use_les:                                            # :195-203
            uc, vc = interpolate_to_cell_center(u, v)
            if les_model == "dynamic_smagorinsky":
                nu_sgs, _ = dynamic_smagorinsky(uc, vc, dx, dy, delta)
            else:
                nu_sgs = constant_smagorinsky(uc, vc, dx, dy, delta, smagorinsky_constant)
        us, vs = rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, U_inf=U_inf, nu_sgs=nu_sgs,
                                     nu_hyper_ratio=nu_hyper_ratio, slip_walls=slip_walls,
                                     fast_mode=fast_mode, brinkman_eta=brinkman_eta,
                                     flow_type=flow_type, advection=advection)
        div = divergence_staggered(us, vs, dx, dy)            # :219-222
        rhs = div / dt
        p = _solve_pressure(rhs, mask, dx, dy, mg, flow_type, mac=True)
        if flow_type in ("von_karman", "lid_driven_cavity"):
            dpx, dpy = grad_x_staggered(p, dx), grad_y_staggered(p, dy)
            if flow_type == "von_karman":
                dpx = dpx.copy()
                dpx[0, :] = 0.0
                dpx = corner_smooth_pressure_gradient(dpx, p.shape[1], 10)
        else:
            dpx, dpy = grad_x_staggered(p, dx), grad_y_staggered(p, dy)
        uc_ = us - dt_correction * dpx
        vc_ = vs - dt_correction * dpy
    else:
        nu_total = nu
        if use_les:                                            # :70-76
            if les_model == "dynamic_smagorinsky":
                nu_sgs, _ = dynamic_smagorinsky(u, v, dx, dy, delta)
            else:
                nu_sgs = constant_smagorinsky(u, v, dx, dy, delta, smagorinsky_constant)
            nu_total = nu + nu_sgs
        us, vs = rk_step_unified(u, v, dt, nu_total, dx, dy, mask, sdf=sdf, U_inf=U_inf,
                                 nu_sgs=nu_sgs, nu_hyper_ratio=nu_hyper_ratio,
                                 slip_walls=slip_walls, fast_mode=fast_mode,
                                 brinkman_eta=brinkman_eta, flow_type=flow_type,
                                 advection=advection)
        if flow_type in ("von_karman", "lid_driven_cavity"):
            div = divergence_nonperiodic(us, vs, dx, dy)
        else:
            div = divergence(us, vs, dx, dy)
        rhs = div / dt                                         # :98
        p = _solve_pressure(rhs, mask, dx, dy, mg, flow_type, mac=False)
        if flow_type == "von_karman":                          # :129-135
            dpx, dpy = grad_x_nonperiodic(p, dx), grad_y_nonperiodic(p, dy)
            dpx = dpx.copy()
            dpx[0, :] = 0.0
            dpx = corner_smooth_pressure_gradient(dpx, p.shape[1], 10)
        else:
            dpx, dpy = grad_x(p, dx), grad_y(p, dy)
        uc_ = us - dt_correction * dpx
        vc_ = vs - dt_correction * dpy
    uc_, vc_ = uc_.copy(), vc_.copy()
    if flow_type == "von_karman":                              # :143-161 / :256-274
        uc_[0, 1:-1] = U_inf
        vc_[0, :] = 0.0
        uc_[-1, :] = uc_[-2, :]
        vc_[-1, :] = vc_[-2, :]
        uc_[:, 0] = 0.0
        uc_[:, -1] = 0.0
        vc_[:, 0] = 0.0
        vc_[:, -1] = 0.0
    elif flow_type == "lid_driven_cavity":
        uc_[:, -1] = U_inf
        vc_[:, -1] = 0.0
        uc_[:, 0] = 0.0
        vc_[:, 0] = 0.0
        uc_[0, :] = 0.0
        vc_[0, :] = 0.0
        uc_[-1, :] = 0.0
        vc_[-1, :] = 0.0
    if grid_type != "mac":                                     # :180-183
        uc_ = np.where(mask > 0.5, uc_, 0.0)
        vc_ = np.where(mask > 0.5, vc_, 0.0)
    if return_nu_sgs:
        return uc_, vc_, p, nu_sgs
    return uc_, vc_, p


# ---------------------------------------------------------------------------
# converging multigrid (new, A17): cell-centred geometric multigrid for the
# reference's own discrete operator, FP64 throughout in this oracle.
# ---------------------------------------------------------------------------
def lap_ref(p, dx, dy):
    """The reference operator (multigrid_solver.py:173-183, edge padding),
    with the outlet row treated as Dirichlet: rows 0..nx-2 are equations,
    row nx-1 is pinned at 0 (:75-77, :194-195)."""
    pp = np.pad(p, ((1, 1), (1, 1)), mode="edge")
    ax, ay = 1.0 / (dx * dx), 1.0 / (dy * dy)
    lap = ax * (pp[2:, 1:-1] + pp[:-2, 1:-1] - 2 * p) + ay * (pp[1:-1, 2:] + pp[1:-1, :-2] - 2 * p)
    lap[-1, :] = 0.0
    return lap


def residual_ref(p, b, dx, dy):
    """r = b - A p on the equation rows; the Dirichlet row carries r = 0."""
    r = b - lap_ref(p, dx, dy)
    r[-1, :] = 0.0
    return r


def rel_residual(p, b, dx, dy):
    """||b - A p||_2 / ||b||_2 over the equation rows, in float64."""
    p = np.asarray(p, np.float64)
    b = np.asarray(b, np.float64).copy()
    b[-1, :] = 0.0
    r = residual_ref(p, b, dx, dy)
    nb = np.sqrt(np.sum(b ** 2))
    return float(np.sqrt(np.sum(r ** 2)) / (nb if nb > 0 else 1.0))


def mg_depth(nx, ny, max_coarse=64):
    """Number of coarsenings: halve while both sizes stay even and the halves
    keep >= 2 cells, until the coarse grid has <= max_coarse cells; always at
    least one coarsening when the grid allows it."""
    k, n, m = 0, nx, ny
    while (n % 2 == 0 and m % 2 == 0 and n // 2 >= 2 and m // 2 >= 2
           and (n * m > max_coarse or k == 0)):
        n, m, k = n // 2, m // 2, k + 1
    return k


def _theta(level):
    """Relative position of the outlet Dirichlet point beyond the last coarse
    cell centre, in units of the coarse spacing: (1 - 2^-l)/2."""
    return 0.5 * (1.0 - 2.0 ** (-level))


def outlet_ghost_factor(level):
    """Ghost value = g * p_last so that the linear interpolant vanishes at the
    fine outlet cell centre; level 0 pins the row instead (g unused)."""
    th = _theta(level)
    return (th - 1.0) / th


def coarse_apply(e, level, dx, dy):
    """Rediscretised operator at level >= 1 (spacing 2^l h): Neumann ghosts on
    the inlet and the walls, outlet ghost g * e_last."""
    hx, hy = dx * 2 ** level, dy * 2 ** level
    ax, ay = 1.0 / hx ** 2, 1.0 / hy ** 2
    ep = np.pad(e, ((1, 1), (1, 1)), mode="edge")
    ep[-1, 1:-1] = outlet_ghost_factor(level) * e[-1, :]
    return ax * (ep[2:, 1:-1] + ep[:-2, 1:-1] - 2 * e) + ay * (ep[1:-1, 2:] + ep[1:-1, :-2] - 2 * e)


def _level_diag(shape, level, dx, dy):
    hx, hy = dx * 2 ** level, dy * 2 ** level
    ax, ay = 1.0 / hx ** 2, 1.0 / hy ** 2
    n, m = shape
    d = np.full(shape, -2.0 * (ax + ay))
    d[0, :] += ax
    d[:, 0] += ay
    d[:, -1] += ay
    if level == 0:
        d[-1, :] += ax          # Neumann-like stencil; the row is pinned anyway
    else:
        d[-1, :] += ax * outlet_ghost_factor(level)
    return d, ax, ay


def rbgs(e, r, level, dx, dy, sweeps, reverse=False):
    """Red-black Gauss-Seidel on A_l e = r (level 0: outlet row pinned)."""
    d, ax, ay = _level_diag(e.shape, level, dx, dy)
    n, m = e.shape
    ii, jj = np.meshgrid(np.arange(n), np.arange(m), indexing="ij")
    colors = (1, 0) if reverse else (0, 1)
    for _ in range(sweeps):
        for c in colors:
            ep = np.pad(e, ((1, 1), (1, 1)), mode="constant")
            nb = ax * (ep[2:, 1:-1] + ep[:-2, 1:-1]) + ay * (ep[1:-1, 2:] + ep[1:-1, :-2])
            e_new = (r - nb) / d
            sel = ((ii + jj) % 2) == c
            if level == 0:
                sel &= ii < n - 1
            e = np.where(sel, e_new, e)
        if level == 0:
            e[-1, :] = 0.0
    return e


def apply_level(e, level, dx, dy):
    if level == 0:
        return lap_ref(e, dx, dy)
    return coarse_apply(e, level, dx, dy)


def restrict_avg(r):
    return 0.25 * (r[0::2, 0::2] + r[1::2, 0::2] + r[0::2, 1::2] + r[1::2, 1::2])


def prolong_bilinear(ec, coarse_level):
    """Cell-centred bilinear prolongation (weights 3/4, 1/4 per axis).
    Ghosts: Neumann copies at inlet and walls; outlet ghost g * e_last."""
    n, m = ec.shape
    g = outlet_ghost_factor(coarse_level)
    ep = np.pad(ec, ((1, 1), (1, 1)), mode="edge")
    ep[-1, 1:-1] = g * ec[-1, :]
    ep[-1, 0] = g * ec[-1, 0]
    ep[-1, -1] = g * ec[-1, -1]
    f = np.zeros((2 * n, 2 * m))
    for di in (0, 1):
        for dj in (0, 1):
            si = -1 if di == 0 else 1
            sj = -1 if dj == 0 else 1
            c0 = ep[1:-1, 1:-1]
            cx = ep[1 + si:n + 1 + si, 1:-1]
            cy = ep[1:-1, 1 + sj:m + 1 + sj]
            cxy = ep[1 + si:n + 1 + si, 1 + sj:m + 1 + sj]
            f[di::2, dj::2] = (9 * c0 + 3 * cx + 3 * cy + cxy) / 16.0
    return f


def coarse_matrix(shape, level, dx, dy):
    """Dense matrix of the coarsest operator (row-major cell order)."""
    n, m = shape
    N = n * m
    A = np.zeros((N, N))
    for k in range(N):
        e = np.zeros(N)
        e[k] = 1.0
        A[:, k] = coarse_apply(e.reshape(n, m), level, dx, dy).ravel()
    return A


def direct_level(nx, ny, depth, max_cells=65536, max_m=128, max_n=1024):
    """Level of the separable direct coarse solve: the first level >= 1 with at
    most max_cells cells, at most max_m cells across and max_n along the
    channel (0: none; the V-cycle then runs down to the dense coarsest grid)."""
    for level in range(1, depth + 1):
        n, m = nx >> level, ny >> level
        if n * m <= max_cells and m <= max_m and n <= max_n and n >= 2:
            return level
    return 0


def _pcr(a, b, c, d):
    """Parallel cyclic reduction of the tridiagonal system (a: sub-, b: main,
    c: super-diagonal) in the arrays' own precision - the GPU's k_cv_dpcr
    schedule (log2 n steps, each eliminating the neighbours at distance st)."""
    a, b, c, d = (x.copy() for x in (a, b, c, d))
    n, st = len(b), 1
    i = np.arange(n)
    while st < n:
        lo, hi = i - st >= 0, i + st < n
        an, cn = np.zeros_like(a), np.zeros_like(c)
        bn, dn = b.copy(), d.copy()
        k1 = a[lo] / b[i[lo] - st]
        an[lo] = -a[i[lo] - st] * k1
        bn[lo] -= c[i[lo] - st] * k1
        dn[lo] -= d[i[lo] - st] * k1
        k2 = c[hi] / b[i[hi] + st]
        cn[hi] = -c[i[hi] + st] * k2
        bn[hi] -= a[i[hi] + st] * k2
        dn[hi] -= d[i[hi] + st] * k2
        a, b, c, d = an, bn, cn, dn
        st *= 2
    return d / b


def coarse_solve_separable(r, level, dx, dy, dtype=np.float64):
    """Exact solve of the level-l operator (level >= 1).  It is separable:
    A = ax Tx (x) I + ay I (x) Ty with Ty the Neumann-Neumann 1-D Laplacian,
    diagonalised by the orthonormal DCT-II (eigenvalues -4 sin^2(pi k/2m)),
    and Tx tridiagonal with an edge ghost at the inlet and the outlet ghost
    g * e_last; one tridiagonal solve in x per cosine mode.
    dtype=np.float32 evaluates the transforms and the parallel cyclic
    reduction in FP32, the precision of the GPU's k_cv_dfwd / k_cv_dpcr /
    k_cv_dbwd."""
    from scipy.linalg import solve_banded
    n, m = r.shape
    hx, hy = dx * 2 ** level, dy * 2 ** level
    ax, ay = 1.0 / hx ** 2, 1.0 / hy ** 2
    kk = np.arange(m)[:, None]
    jj = np.arange(m)[None, :]
    C = np.sqrt(2.0 / m) * np.cos(np.pi * kk * (2 * jj + 1) / (2.0 * m))
    C[0, :] = np.sqrt(1.0 / m)
    ly = -4.0 * ay * np.sin(np.pi * np.arange(m) / (2.0 * m)) ** 2
    dxv = np.full(n, -2.0)
    dxv[0] += 1.0
    dxv[-1] += outlet_ghost_factor(level)
    if dtype == np.float32:
        f = np.float32
        C32 = C.astype(f)
        rh = r.astype(f) @ C32.T
        eh = np.empty_like(rh)
        sub = np.full(n, ax, f)
        sub[0] = 0
        sup = np.full(n, ax, f)
        sup[-1] = 0
        for k in range(m):
            eh[:, k] = _pcr(sub, (ax * dxv + ly[k]).astype(f), sup, rh[:, k])
        return (eh @ C32).astype(np.float64)
    rh = r @ C.T
    eh = np.empty_like(rh)
    for k in range(m):
        ab = np.zeros((3, n))
        ab[0, 1:] = ax
        ab[1] = ax * dxv + ly[k]
        ab[2, :-1] = ax
        eh[:, k] = solve_banded((1, 1), ab, rh[:, k])
    return eh @ C


def v_cycle_converge(r, dx, dy, depth, nu1=2, nu2=2, direct=0, coarse_dtype=np.float64,
                     nu2_fine=1):
    """One V(nu1,nu2) cycle for A e = r from e = 0; returns e (level 0).
    The finest level post-smooths with nu2_fine sweeps (the GPU's k_cv_up0:
    one red-black sweep, a V(2,1) cycle on the fine grid).  With direct > 0
    the cycle stops at that level with the separable exact solve (in
    coarse_dtype); else it descends to the dense coarsest grid."""
    def cyc(rl, level):
        if direct and level == direct:
            return coarse_solve_separable(rl, level, dx, dy, coarse_dtype)
        if level == depth:
            A = coarse_matrix(rl.shape, level, dx, dy)
            return np.linalg.solve(A, rl.ravel()).reshape(rl.shape)
        e = rbgs(np.zeros_like(rl), rl, level, dx, dy, nu1)
        res = rl - apply_level(e, level, dx, dy)
        if level == 0:
            res[-1, :] = 0.0
        ec = cyc(restrict_avg(res), level + 1)
        e = e + prolong_bilinear(ec, level + 1)
        if level == 0:
            e[-1, :] = 0.0
        return rbgs(e, rl, level, dx, dy, nu2_fine if level == 0 else nu2)
    return cyc(r, 0)


def mg_converge(b, dx, dy, rtol=1e-6, max_cycles=40, p0=None, nu1=2, nu2=2, max_coarse=64,
                direct=True, coarse_dtype=np.float64, nu2_fine=1):
    """Converging mode: iterative refinement around V-cycles.  Each outer
    iteration computes r = b - A p in float64, runs one V-cycle on A e = r and
    adds e.  Stops when ||r||/||b|| <= rtol.  Returns (p, info).  The V-cycle
    ends in the separable direct solve at direct_level() when direct is True
    (as on the GPU), else at the dense coarsest grid; coarse_dtype selects the
    precision of that direct solve."""
    b = np.asarray(b, np.float64).copy()
    b[-1, :] = 0.0
    nx, ny = b.shape
    depth = mg_depth(nx, ny, max_coarse)
    dlev = direct_level(nx, ny, depth) if direct else 0
    p = np.zeros_like(b) if p0 is None else np.asarray(p0, np.float64).copy()
    p[-1, :] = 0.0
    nb = np.sqrt(np.sum(b ** 2))
    nb = nb if nb > 0 else 1.0
    hist = []
    cycles = 0
    while True:
        r = residual_ref(p, b, dx, dy)
        rel = np.sqrt(np.sum(r ** 2)) / nb
        hist.append(float(rel))
        if rel <= rtol or cycles >= max_cycles:
            break
        p = p + v_cycle_converge(r, dx, dy, depth, nu1, nu2, dlev, coarse_dtype, nu2_fine)
        p[-1, :] = 0.0
        cycles += 1
    return p, {"cycles": cycles, "rel_residual": hist[-1], "history": hist, "depth": depth,
               "direct_level": dlev}


# ---------------------------------------------------------------------------
# geometry — solver/simulation/mask_generator.py, obstacles/*.py
# ---------------------------------------------------------------------------
def grid_coords(nx, ny, lx, ly):
    """solver/params.py:51-56: dx = lx/nx but coordinates are
    linspace(0, lx, nx) (so cell i sits at i*lx/(nx-1))."""
    x = np.linspace(0, lx, nx)
    y = np.linspace(0, ly, ny)
    return np.meshgrid(x, y, indexing="ij")


def sdf_cylinder(X, Y, cx, cy, r):
    """mask_generator.py:151-153."""
    return np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r


def sdf_three_cylinders_inline(X, Y, cx, cy, diameter, spacing):
    """obstacles/cylinder_array.py:8-42 (three cylinders in a row along x)."""
    r = diameter / 2.0
    s1 = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r
    s2 = np.sqrt((X - (cx + spacing)) ** 2 + (Y - cy) ** 2) - r
    s3 = np.sqrt((X - (cx + 2 * spacing)) ** 2 + (Y - cy) ** 2) - r
    return np.minimum(np.minimum(s1, s2), s3)


def triangle_centres(cx, cy, spacing):
    """Three centres on an equilateral triangle of side ``spacing`` whose
    centroid is (cx, cy), apex pointing upstream (new geometry)."""
    R = spacing / math.sqrt(3.0)
    return [(cx - R, cy),
            (cx + 0.5 * R, cy + 0.5 * spacing),
            (cx + 0.5 * R, cy - 0.5 * spacing)]


def sdf_three_cylinders_triangle(X, Y, cx, cy, diameter, spacing):
    r = diameter / 2.0
    s = None
    for (px, py) in triangle_centres(cx, cy, spacing):
        d = np.sqrt((X - px) ** 2 + (Y - py) ** 2) - r
        s = d if s is None else np.minimum(s, d)
    return s


def sdf_naca4(X, Y, chord, aoa_deg, px, py, m, p, t):
    """obstacles/naca_airfoils.py:109-178 (the camber branch of a symmetric
    section divides 0/0 at x<=0, exactly as the reference does; those points
    are outside the chord and never selected)."""
    m, p, t = np.float64(m), np.float64(p), np.float64(t)
    with np.errstate(divide="ignore", invalid="ignore"):
        Xl, Yl = X - px, Y - py
        a = np.radians(aoa_deg)
        Xr = Xl * np.cos(a) - Yl * np.sin(a)
        Yr = Xl * np.sin(a) + Yl * np.cos(a)
        xn, yn = Xr / chord, Yr / chord
        inc = (xn >= 0) & (xn <= 1)
        xs = np.clip(xn, 0.0, 1.0)
        yt = 5 * t * (0.2969 * np.sqrt(np.abs(xs)) - 0.1260 * xs - 0.3516 * xs ** 2
                      + 0.2843 * xs ** 3 - 0.1015 * xs ** 4)
        yc = np.where(xn <= p, m / p ** 2 * (2 * p * xn - xn ** 2),
                      m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * xn - xn ** 2))
        dyc = np.where(xn <= p, 2 * m / p ** 2 * (p - xn), 2 * m / (1 - p) ** 2 * (p - xn))
        th = np.arctan(dyc)
        yu = yc + yt * np.cos(th)
        yl = yc - yt * np.cos(th)
        dist_s = np.minimum(np.abs(yn - yu) * chord, np.abs(yn - yl) * chord)
        dle = np.sqrt(Xr ** 2 + Yr ** 2)
        dte = np.sqrt((Xr - chord) ** 2 + Yr ** 2)
        dist = np.where(inc, dist_s, np.minimum(dle, dte))
        inside = inc & (yn >= yl - 0.01) & (yn <= yu + 0.01)
        return np.where(inside, -dist, dist)


def mask_from_sdf(sdf, eps):
    """mask_generator.py:155-158: mask = 1 - sigmoid(-sdf/eps)."""
    return 1.0 - sigmoid(-sdf / eps)


# ---------------------------------------------------------------------------
# the Re presets — solver/params.py:233-254, 308-413
# ---------------------------------------------------------------------------
def compute_eps_multiplier(Re):
    if Re <= 1000:
        return 0.05
    if Re <= 2000:
        return 0.05
    if Re <= 5000:
        return 0.03
    return 0.02


def get_re_parameters(Re, grid_nx=512):
    p = {"C_s": 0.1, "nu_hyper_ratio": 0.0, "brinkman_eta": 1e-4, "dt_max": 0.01,
         "cfl_target": 0.3, "nu_h": 0.0}
    table = [
        (1000, 0.08, 0.0, 1e-4, 0.005, 0.3, 0.0),
        (10000, 0.1, 0.01, 1e-4, 0.008, 0.25, 0.0),
        (100000, 0.12, 0.03, 1e-6, 0.008, 0.35, 0.0),
        (1000000, 0.15, 0.05, 1e-7, 0.006, 0.3, 1e-5),
        (10000000, 0.18, 0.08, 1e-7, 0.004, 0.25, 2e-5),
    ]
    for lim, cs, hr, eta, dtm, cfl, nuh in table:
        if Re <= lim:
            p.update(C_s=cs, nu_hyper_ratio=hr, brinkman_eta=eta, dt_max=dtm, cfl_target=cfl, nu_h=nuh)
            break
    else:
        p.update(C_s=0.20, nu_hyper_ratio=0.1, brinkman_eta=1e-7, dt_max=0.003, cfl_target=0.2, nu_h=3e-5)
    if grid_nx < 512:
        p["C_s"] *= 1.2
        p["nu_hyper_ratio"] *= 1.5
        p["brinkman_eta"] *= 1.2
        p["cfl_target"] *= 0.8
    return p
