"""Reverse mode (vector-Jacobian product) of the collocated step_pure, in
NumPy FP64.  TEST INFRASTRUCTURE ONLY: the GPU adjoint (aj_step_vjp) is
checked against this; nothing on the product path imports it.

What it differentiates is what ``jax.grad`` differentiates in the reference's
rollouts: solver/solver.py:34-75 (differentiable_rollout: lax.scan over
step_pure) and :78-114 (design_loss / grad_design_loss, gradients with
respect to the params dict: the SDF, nu, U_inf).  The step is
solver/pure_functions/step.py:49-467 on the collocated grid with the
von Karman boundary conditions, first-order upwind RK3 (or RK2) with the
implicit Brinkman term (advection_schemes/rk3_simple_new.py:175-358) and the
parity multigrid (pressure_solvers/multigrid_solver.py:55-241).  JAX's rules
are reproduced where they matter: ``where(c, x, y)`` passes the cotangent to
the selected branch only (the condition has no derivative), array updates
``.at[...].set`` drop the cotangent of the overwritten entries, and
``lax.cond`` inside the V-cycle scan differentiates only the branch taken,
so the adjoint runs as many V-cycles as the forward did.

Pinned by finite differences of the pinned forward (oracle.ref_np.step_pure,
itself pinned to golden vectors of the reference): the directional
derivative of <g, step(x)> matches <vjp(g), direction> (tests).
"""
from __future__ import annotations

import numpy as np

from . import ref_np as R

__all__ = ["step_pure_vjp", "step_gui_vjp", "forward_stages", "mg_vjp", "rollout",
           "rollout_vjp"]


# ------------------------------------------------------------------ pieces
def _lap(f, dx, dy):
    """Edge-padded 5-point Laplacian (rk3_simple_new.py:215-219); symmetric,
    so it is its own transpose."""
    fp = np.pad(f, ((1, 1), (1, 1)), mode="edge")
    return ((fp[2:, 1:-1] + fp[:-2, 1:-1] - 2 * f) / dx ** 2
            + (fp[1:-1, 2:] + fp[1:-1, :-2] - 2 * f) / dy ** 2)


def _one_sided(f, vel, h, axis):
    """The upwind difference of rk3_simple_new.py:287-298 along ``axis``:
    (f - f_prev)/h where vel > 0, else (f_next - f)/h, edge-padded."""
    pw = [(0, 0), (0, 0)]
    pw[axis] = (1, 1)
    fp = np.pad(f, pw, mode="edge")
    n = f.shape[axis]
    prev = np.take(fp, np.arange(0, n), axis=axis)
    nxt = np.take(fp, np.arange(2, n + 2), axis=axis)
    return np.where(vel > 0, (f - prev) / h, (nxt - f) / h)


def _one_sided_T(alpha, vel, h, axis):
    """Transpose of f -> _one_sided(f, vel, h, axis) applied to alpha (vel
    fixed).  Row c with vel > 0 reads +f[c] - f[prev(c)], otherwise
    -f[c] + f[next(c)]; prev/next clamp at the edges."""
    a = np.moveaxis(alpha / h, axis, 0)
    pos = np.moveaxis(vel > 0, axis, 0)
    out = np.where(pos, a, -a)
    ap = np.where(pos, a, 0.0)          # -a goes to prev(c)
    an = np.where(pos, 0.0, a)          # +a goes to next(c)
    out[:-1] -= ap[1:]
    out[0] -= ap[0]
    out[1:] += an[:-1]
    out[-1] += an[-1]
    return np.moveaxis(out, 0, axis)


def _rhs(u, v, nu, dx, dy, hyper=0.0):
    """compute_rhs_explicit (rk3_simple_new.py:284-313) without LES: upwind
    advection, nu * Laplacian and, with ``hyper`` (nu_hyper_ratio) > 0, the
    bi-Laplacian term nu * hyper * dx * dy * lap(lap(w)) (:307-312, sponge
    disabled)."""
    adv_u = u * _one_sided(u, u, dx, 0) + v * _one_sided(u, v, dy, 1)
    adv_v = u * _one_sided(v, u, dx, 0) + v * _one_sided(v, v, dy, 1)
    lu, lv = _lap(u, dx, dy), _lap(v, dx, dy)
    ru, rv = -adv_u + nu * lu, -adv_v + nu * lv
    if hyper > 0:
        nh = nu * hyper * (dx * dy)
        ru = ru - nh * _lap(lu, dx, dy)
        rv = rv - nh * _lap(lv, dx, dy)
    return ru, rv


def _rhs_T(ku_bar, kv_bar, u, v, nu, dx, dy, hyper=0.0):
    """Cotangents of (u, v) from cotangents of _rhs(u, v), and d/d nu (the
    Laplacian and its square are symmetric, so each is its own transpose)."""
    a, b = -ku_bar, -kv_bar                          # cotangents of adv_u, adv_v
    fxu, fyu = _one_sided(u, u, dx, 0), _one_sided(u, v, dy, 1)
    fxv, fyv = _one_sided(v, u, dx, 0), _one_sided(v, v, dy, 1)
    ub = nu * _lap(ku_bar, dx, dy)
    vb = nu * _lap(kv_bar, dx, dy)
    if hyper > 0:
        nh = nu * hyper * (dx * dy)
        ub = ub - nh * _lap(_lap(ku_bar, dx, dy), dx, dy)
        vb = vb - nh * _lap(_lap(kv_bar, dx, dy), dx, dy)
    # velocity roles
    ub += a * fxu + b * fxv
    vb += a * fyu + b * fyv
    # field roles (velocities fixed)
    ub += _one_sided_T(a * u, u, dx, 0) + _one_sided_T(a * v, v, dy, 1)
    vb += _one_sided_T(b * u, u, dx, 0) + _one_sided_T(b * v, v, dy, 1)
    tu, tv = ku_bar * _lap(u, dx, dy), kv_bar * _lap(v, dx, dy)
    if hyper > 0:
        hh = hyper * (dx * dy)
        tu = tu - hh * ku_bar * _lap(_lap(u, dx, dy), dx, dy)
        tv = tv - hh * kv_bar * _lap(_lap(v, dx, dy), dx, dy)
    nu_bar = float(np.sum(tu) + np.sum(tv))
    nu_abs = float(np.sum(np.abs(tu)) + np.sum(np.abs(tv)))   # the sum's magnitude scale
    return ub, vb, nu_bar, nu_abs


def _bc_T(gu, gv, slip=True):
    """Transpose of the von Karman slip-wall boundary conditions
    (rk3_simple_new.py:262-275 and step.py:365-377, the same statements):
    u[0]=U, v[0]=0, u[-1]=u[-2], v[-1]=v[-2], u[:,0]=u[:,1], u[:,-1]=u[:,-2],
    v[:,0]=0, v[:,-1]=0, undone in reverse order.  Returns the cotangent of
    U_inf as well, and the sum of the magnitudes it adds up."""
    gu, gv = gu.copy(), gv.copy()
    gv[:, -1] = 0.0
    gv[:, 0] = 0.0
    if slip:
        gu[:, -2] += gu[:, -1]
        gu[:, 1] += gu[:, 0]
    gu[:, -1] = 0.0                                   # (no-slip: u = 0 on the walls)
    gu[:, 0] = 0.0
    gv[-2, :] += gv[-1, :]
    gv[-1, :] = 0.0
    gu[-2, :] += gu[-1, :]
    gu[-1, :] = 0.0
    gv[0, :] = 0.0
    U_bar = float(np.sum(gu[0, :]))
    U_abs = float(np.sum(np.abs(gu[0, :])))
    gu[0, :] = 0.0
    return gu, gv, U_bar, U_abs


def _bc_gui_T(gu, gv):
    """Transpose of the GUI step's boundary rows (step_handlers.py:143-161):
    u[0, 1:-1] = U, v[0] = 0, u[-1] = u[-2], v[-1] = v[-2], u and v zero on
    both walls, undone in reverse order."""
    gu, gv = gu.copy(), gv.copy()
    gv[:, -1] = 0.0
    gv[:, 0] = 0.0
    gu[:, -1] = 0.0
    gu[:, 0] = 0.0
    gv[-2, :] += gv[-1, :]
    gv[-1, :] = 0.0
    gu[-2, :] += gu[-1, :]
    gu[-1, :] = 0.0
    gv[0, :] = 0.0
    U_bar = float(np.sum(gu[0, 1:-1]))
    U_abs = float(np.sum(np.abs(gu[0, 1:-1])))
    gu[0, 1:-1] = 0.0
    return gu, gv, U_bar, U_abs


def _bc_inlet_T(gu, gv):
    """Transpose of step.py:182-191 (applied to the predictor output):
    us[0]=U, vs[0]=0, us[:,0]=us[:,1], us[:,-1]=us[:,-2], vs[:,0]=vs[:,-1]=0."""
    gu, gv = gu.copy(), gv.copy()
    gv[:, -1] = 0.0
    gv[:, 0] = 0.0
    gu[:, -2] += gu[:, -1]
    gu[:, -1] = 0.0
    gu[:, 1] += gu[:, 0]
    gu[:, 0] = 0.0
    gv[0, :] = 0.0
    U_bar = float(np.sum(gu[0, :]))
    U_abs = float(np.sum(np.abs(gu[0, :])))
    gu[0, :] = 0.0
    return gu, gv, U_bar, U_abs


def _gx_T(g, dx):
    """Transpose of grad_x_nonperiodic (operators.py:17-32)."""
    f = np.zeros_like(g)
    f[2:, :] += g[1:-1, :] / (2.0 * dx)
    f[:-2, :] -= g[1:-1, :] / (2.0 * dx)
    f[1, :] += g[0, :] / dx
    f[0, :] -= g[0, :] / dx
    f[-1, :] += g[-1, :] / dx
    f[-2, :] -= g[-1, :] / dx
    return f


def _gy_T(g, dy):
    return _gx_T(g.T, dy).T


def _div_T(d, dx, dy):
    """Transpose of divergence_nonperiodic (operators.py:81-96)."""
    ub, vb = np.zeros_like(d), np.zeros_like(d)
    di = d[1:-1, 1:-1]
    ub[2:, 1:-1] += di / (2.0 * dx)
    ub[:-2, 1:-1] -= di / (2.0 * dx)
    vb[1:-1, 2:] += di / (2.0 * dy)
    vb[1:-1, :-2] -= di / (2.0 * dy)
    return ub, vb


# ------------------------------------------------------------------ multigrid
def _smooth_T(pbar, k, ax, ay):
    """Transpose of k Jacobi sweeps p <- (N p - b)/d with edge ghosts
    (multigrid_solver.py:158-171).  N (neighbour sum with edge ghosts) is
    symmetric, so each reversed sweep is h = pbar/d, b_bar -= h,
    pbar = N h.  Returns (cotangent of the sweeps' input p, of b)."""
    d = 2.0 * (ax + ay)
    bbar = np.zeros_like(pbar)
    for _ in range(k):
        h = pbar / d
        bbar -= h
        hp = np.pad(h, ((1, 1), (1, 1)), mode="edge")
        pbar = ax * (hp[2:, 1:-1] + hp[:-2, 1:-1]) + ay * (hp[1:-1, 2:] + hp[1:-1, :-2])
    return pbar, bbar


def _restrict_T(rc):
    """Transpose of the unscaled 2x2 average (multigrid_solver.py:108-132)."""
    return 0.25 * np.repeat(np.repeat(rc, 2, axis=0), 2, axis=1)


def _prolong_T(f):
    """Transpose of the reference prolongation (multigrid_solver.py:134-156):
    injection at even indices, averages at interior odd ones, the last fine
    row and column zero."""
    n, m = f.shape[0] // 2, f.shape[1] // 2
    c = f[::2, ::2].copy()
    if 2 * n > 2:
        h = 0.5 * f[1:-1:2, ::2]                 # rows 2I+1, I = 0..n-2
        c[:-1, :] += h
        c[1:, :] += h
    if 2 * m > 2:
        h = 0.5 * f[::2, 1:-1:2]
        c[:, :-1] += h
        c[:, 1:] += h
    if 2 * n > 2 and 2 * m > 2:
        h = 0.25 * f[1:-1:2, 1:-1:2]
        c[:-1, :-1] += h
        c[1:, :-1] += h
        c[:-1, 1:] += h
        c[1:, 1:] += h
    return c


def mg_vjp(pbar, dx, dy, levels=4, cycles=1):
    """Cotangent of the rhs of R.poisson_multigrid (collocated, von Karman,
    zero initial guess) from the cotangent of its result, for ``cycles``
    V-cycles run (multigrid_solver.py:173-241)."""
    nx, ny = pbar.shape
    max_levels = R.mg_levels_ok(nx, ny, levels)
    ax, ay = 1.0 / dx ** 2, 1.0 / dy ** 2

    def lap_edge(p):
        pp = np.pad(p, ((1, 1), (1, 1)), mode="edge")
        return ax * (pp[2:, 1:-1] + pp[:-2, 1:-1] - 2 * p) + ay * (pp[1:-1, 2:] + pp[1:-1, :-2] - 2 * p)

    def cyc_T(p3, level):
        if level >= max_levels:
            return _smooth_T(p3, 10, ax, ay)
        p3 = p3.copy()
        p3[-1, :] = 0.0                               # p.at[-1].set(0) after post-smoothing
        p2, bbar = _smooth_T(p3, 2, ax, ay)
        ec = _prolong_T(p2)
        _, rc_bar = cyc_T(ec, level + 1)              # coarse guess is zero
        r_bar = _restrict_T(rc_bar)
        bbar = bbar + r_bar
        p1 = p2 - lap_edge(r_bar)                     # r = b - A p1, A symmetric
        p1[-1, :] = 0.0                               # after pre-smoothing
        p0, b2 = _smooth_T(p1, 2, ax, ay)
        return p0, bbar + b2

    b_bar = np.zeros_like(pbar)
    for _ in range(cycles):
        pbar, bc = cyc_T(pbar, 0)
        b_bar += bc
    b_bar[-1, :] = 0.0                                # b.at[-1].set(0)
    return b_bar


# ------------------------------------------------------------------ the step
def _chi(mask, sdf, dx):
    return R.sigmoid(-sdf / (0.1 * dx)) if sdf is not None else 1.0 - mask


def forward_stages(u, v, dt, mask, sdf, dx, dy, nu, U_inf, fast_mode=False, brinkman_eta=0.005,
                   hyper=0.0):
    """The predictor of step_pure with its stage states kept: returns
    (stages, (us, vs)), stages = list of (u_k, v_k) fed to compute_rhs_explicit
    and the pre-mask final combination."""
    chi = _chi(mask, sdf, dx)
    den = 1 + dt * chi / brinkman_eta
    k1u, k1v = _rhs(u, v, nu, dx, dy, hyper)
    if not fast_mode:
        u2, v2 = (u + dt * k1u) / den, (v + dt * k1v) / den
        k2u, k2v = _rhs(u2, v2, nu, dx, dy, hyper)
        u3 = (0.75 * u + 0.25 * (u + dt * k2u)) / den
        v3 = (0.75 * v + 0.25 * (v + dt * k2v)) / den
        k3u, k3v = _rhs(u3, v3, nu, dx, dy, hyper)
        un = ((1 / 3) * u + (2 / 3) * (u + dt * k3u)) / den
        vn = ((1 / 3) * v + (2 / 3) * (v + dt * k3v)) / den
        stages = [(u, v), (u2, v2), (u3, v3)]
    else:
        u2, v2 = (u + dt * k1u) / den, (v + dt * k1v) / den
        k2u, k2v = _rhs(u2, v2, nu, dx, dy, hyper)
        un = (u + 0.5 * dt * (k1u + k2u)) / den
        vn = (v + 0.5 * dt * (k1v + k2v)) / den
        stages = [(u, v), (u2, v2)]
    return stages, (un, vn), den, chi


def step_pure_vjp(u, v, dt, mask, sdf, dx, dy, nu, U_inf, gu, gv, gp=None, *, v_cycles=1,
                  levels=4, fast_mode=False, brinkman_eta=0.005):
    """Cotangents of step_pure's inputs from cotangents (gu, gv, gp) of its
    outputs (u_new, v_new, p).  Returns a dict: u, v (fields), sdf (field, or
    None without an SDF: chi = 1 - mask then), nu, U_inf (floats), and the
    forward outputs under 'out'."""
    u, v, mask = (np.asarray(a, np.float64) for a in (u, v, mask))
    sdf = None if sdf is None else np.asarray(sdf, np.float64)
    gu, gv = np.asarray(gu, np.float64), np.asarray(gv, np.float64)
    nx, ny = u.shape
    gp = np.zeros((nx, ny)) if gp is None else np.asarray(gp, np.float64)
    live = mask > 0.5

    # ---- forward, keeping what the reverse pass reads
    stages, (un_pre, vn_pre), den, chi = forward_stages(u, v, dt, mask, sdf, dx, dy, nu, U_inf,
                                                        fast_mode, brinkman_eta)
    us = np.where(live, un_pre, 0.0)
    vs = np.where(live, vn_pre, 0.0)
    us, vs = R.bc_collocated(us, vs, U_inf, "von_karman", True)
    us, vs = us.copy(), vs.copy()                              # step.py:182-191
    us[0, :] = U_inf
    vs[0, :] = 0.0
    us[:, 0] = us[:, 1]
    us[:, -1] = us[:, -2]
    vs[:, 0] = 0.0
    vs[:, -1] = 0.0
    div = R.divergence_nonperiodic(us, vs, dx, dy)
    rhs = (div * mask) / dt
    p, info = R.poisson_multigrid(rhs, mask, dx, dy, levels, v_cycles, 1e-6, "von_karman",
                                  return_info=True)
    dmx, dmy = R.grad_x_nonperiodic(mask, dx), R.grad_y_nonperiodic(mask, dy)
    gm = np.sqrt(dmx ** 2 + dmy ** 2)
    iface = gm > 0.1 / dx
    nxv, nyv = dmx / (gm + 1e-8), dmy / (gm + 1e-8)

    U_bar = 0.0
    # ---- correction (step.py:259-397), reversed
    g_u = np.where(live, gu, 0.0)                               # :396-397
    g_v = np.where(live, gv, 0.0)
    g_u, g_v, ub, ua = _bc_T(g_u, g_v)                          # :365-377
    U_bar += ub
    U_abs = ua
    g_u = np.where(live, g_u, 0.0)                              # :348-349
    g_v = np.where(live, g_v, 0.0)
    us_bar, vs_bar = g_u.copy(), g_v.copy()
    dpx_bar, dpy_bar = -dt * g_u, -dt * g_v
    dpx_bar[0, :] = 0.0                                         # :341
    dn_bar = -(dpx_bar * nxv + dpy_bar * nyv)                   # :313-335
    dpx_bar = np.where(iface, dpx_bar + dn_bar * nxv, dpx_bar)
    dpy_bar = np.where(iface, dpy_bar + dn_bar * nyv, dpy_bar)
    p_bar = gp + _gx_T(dpx_bar, dx) + _gy_T(dpy_bar, dy)
    # ---- pressure solve, rhs and divergence (step.py:182-199), reversed
    rhs_bar = mg_vjp(p_bar, dx, dy, levels, info["cycles"])
    div_bar = rhs_bar * mask / dt
    dub, dvb = _div_T(div_bar, dx, dy)
    us_bar += dub
    vs_bar += dvb
    us_bar, vs_bar, ub, ua = _bc_inlet_T(us_bar, vs_bar)
    U_bar += ub
    U_abs += ua
    # ---- predictor, reversed
    g = _predictor_T(us_bar, vs_bar, stages, (un_pre, vn_pre), den, chi, live, dt, nu, dx, dy,
                     fast_mode, 0.0, True, sdf is not None, brinkman_eta)
    U_bar += g["U_inf"]
    U_abs += g["U_inf_abs"]
    # forward outputs (for callers and tests)
    un, vn, pp = R.step_pure(u, v, dt, mask, sdf, dx, dy, nu, U_inf, v_cycles=v_cycles,
                             fast_mode=fast_mode, brinkman_eta=brinkman_eta,
                             mg=R.MGConfig(mode="parity", v_cycles=v_cycles, levels=levels))
    return {"u": g["u"], "v": g["v"], "sdf": g["sdf"], "nu": g["nu"], "U_inf": U_bar,
            "nu_abs": g["nu_abs"], "U_inf_abs": U_abs, "cycles": info["cycles"],
            "out": (un, vn, pp)}


def _predictor_T(us_bar, vs_bar, stages, wn, den, chi, live, dt, nu, dx, dy, fast_mode, hyper,
                 slip, has_sdf, brinkman_eta):
    """Reverse of rk_step_unified (rk3_simple_new.py:315-358) from the
    cotangent of its output (after its hard mask and boundary rows): the
    cotangents of its inputs u, v, of the SDF through chi (has_sdf), of nu
    and of U_inf (the inlet row it sets)."""
    us_bar, vs_bar, U_bar, U_abs = _bc_T(us_bar, vs_bar, slip)
    un_pre, vn_pre = wn
    xu = np.where(live, us_bar, 0.0) / den
    xv = np.where(live, vs_bar, 0.0) / den
    den_bar = -(xu * un_pre + xv * vn_pre)
    nu_bar = nu_abs = 0.0

    def rT(ku, kv, uu, vv):
        nonlocal nu_bar, nu_abs
        a, b, nb, na = _rhs_T(ku, kv, uu, vv, nu, dx, dy, hyper)
        nu_bar += nb
        nu_abs += na
        return a, b

    if not fast_mode:
        (u1, v1), (u2, v2), (u3, v3) = stages
        w1u, w1v = xu.copy(), xv.copy()                         # (1/3 + 2/3) of x_n
        a, b = rT((2 / 3) * dt * xu, (2 / 3) * dt * xv, u3, v3)
        xu, xv = a / den, b / den
        den_bar -= xu * u3 + xv * v3
        w1u += xu                                               # 0.75 + 0.25
        w1v += xv
        a, b = rT(0.25 * dt * xu, 0.25 * dt * xv, u2, v2)
        xu, xv = a / den, b / den
        den_bar -= xu * u2 + xv * v2
        w1u += xu
        w1v += xv
        ku, kv = dt * xu, dt * xv
    else:
        (u1, v1), (u2, v2) = stages
        w1u, w1v = xu.copy(), xv.copy()
        k1u, k1v = 0.5 * dt * xu, 0.5 * dt * xv
        a, b = rT(0.5 * dt * xu, 0.5 * dt * xv, u2, v2)
        xu, xv = a / den, b / den
        den_bar -= xu * u2 + xv * v2
        w1u += xu
        w1v += xv
        ku, kv = k1u + dt * xu, k1v + dt * xv
    a, b = rT(ku, kv, u1, v1)
    sdf_bar = None
    if has_sdf:
        chi_bar = den_bar * dt / brinkman_eta
        sdf_bar = chi_bar * chi * (1.0 - chi) * (-1.0 / (0.1 * dx))
    return {"u": w1u + a, "v": w1v + b, "sdf": sdf_bar, "nu": nu_bar, "nu_abs": nu_abs,
            "U_inf": U_bar, "U_inf_abs": U_abs}


def step_gui_vjp(u, v, dt, mask, sdf, dx, dy, nu, U_inf, gu, gv, gp=None, *, v_cycles=5,
                 levels=4, fast_mode=False, brinkman_eta=1e-4, nu_hyper_ratio=0.0,
                 slip_walls=True):
    """Reverse mode of the collocated GUI step without LES
    (step_handlers.py:62-185: BaselineSolver._step, which the WIP optimizer
    scans under jax.grad, inverse_design_WIP/optimizer_autodiff.py:113-205).
    Differences from step_pure: hyperviscosity and the wall condition are
    options of the predictor, rhs = div/dt (no mask), the correction has no
    interface projection, its boundary rows exclude the inlet corners and
    hold u = v = 0 on the walls, one hard mask at the end.  The corner
    smoothing of the gradient (corner_smoothing.py:39-61) scales a row that
    was just zeroed, so it adds nothing.  Same return value as
    step_pure_vjp."""
    u, v, mask = (np.asarray(a, np.float64) for a in (u, v, mask))
    sdf = None if sdf is None else np.asarray(sdf, np.float64)
    gu, gv = np.asarray(gu, np.float64), np.asarray(gv, np.float64)
    nx, ny = u.shape
    gp = np.zeros((nx, ny)) if gp is None else np.asarray(gp, np.float64)
    live = mask > 0.5
    stages, (un_pre, vn_pre), den, chi = forward_stages(u, v, dt, mask, sdf, dx, dy, nu, U_inf,
                                                        fast_mode, brinkman_eta, nu_hyper_ratio)
    us = np.where(live, un_pre, 0.0)
    vs = np.where(live, vn_pre, 0.0)
    us, vs = R.bc_collocated(us, vs, U_inf, "von_karman", slip_walls)
    rhs = R.divergence_nonperiodic(us, vs, dx, dy) / dt
    p, info = R.poisson_multigrid(rhs, mask, dx, dy, levels, v_cycles, 1e-6, "von_karman",
                                  return_info=True)
    # ---- correction (step_handlers.py:128-183), reversed
    g_u = np.where(live, gu, 0.0)
    g_v = np.where(live, gv, 0.0)
    g_u, g_v, U_bar, U_abs = _bc_gui_T(g_u, g_v)
    us_bar, vs_bar = g_u.copy(), g_v.copy()
    dpx_bar, dpy_bar = -dt * g_u, -dt * g_v
    dpx_bar[0, :] = 0.0                                         # :134-135
    p_bar = gp + _gx_T(dpx_bar, dx) + _gy_T(dpy_bar, dy)
    # ---- pressure solve, rhs and divergence (:92-98), reversed
    rhs_bar = mg_vjp(p_bar, dx, dy, levels, info["cycles"])
    dub, dvb = _div_T(rhs_bar / dt, dx, dy)
    us_bar += dub
    vs_bar += dvb
    g = _predictor_T(us_bar, vs_bar, stages, (un_pre, vn_pre), den, chi, live, dt, nu, dx, dy,
                     fast_mode, nu_hyper_ratio, slip_walls, sdf is not None, brinkman_eta)
    un, vn, pp = R.step_gui(u, v, mask, dt, sdf=sdf, dx=dx, dy=dy, nu=nu, U_inf=U_inf,
                            nu_hyper_ratio=nu_hyper_ratio, slip_walls=slip_walls,
                            fast_mode=fast_mode, brinkman_eta=brinkman_eta, v_cycles=v_cycles,
                            mg=R.MGConfig(mode="parity", v_cycles=v_cycles, levels=levels))
    return {"u": g["u"], "v": g["v"], "sdf": g["sdf"], "nu": g["nu"],
            "U_inf": U_bar + g["U_inf"], "nu_abs": g["nu_abs"], "U_inf_abs": U_abs + g["U_inf_abs"],
            "cycles": info["cycles"], "out": (un, vn, pp)}


# ------------------------------------------------------------------ rollouts
def rollout(u, v, dt, mask, sdf, dx, dy, nu, U_inf, num_steps, **kw):
    """differentiable_rollout (solver/solver.py:34-75): the final state and
    the history of (u, v) after every step (lax.scan's stacked output)."""
    hist = []
    for _ in range(num_steps):
        u, v, _ = R.step_pure(u, v, dt, mask, sdf, dx, dy, nu, U_inf, **kw)
        hist.append((u, v))
    return (u, v), hist


def rollout_vjp(u0, v0, dt, mask, sdf, dx, dy, nu, U_inf, num_steps, gu, gv, *, v_cycles=1,
                fast_mode=False, brinkman_eta=0.005):
    """Cotangents of the rollout's initial (u, v), SDF, nu and U_inf from the
    cotangent of its final (u, v): the reverse scan, one step_pure_vjp per
    step from the stored inputs."""
    states = [(np.asarray(u0, np.float64), np.asarray(v0, np.float64))]
    for _ in range(num_steps - 1):
        u, v, _ = R.step_pure(*states[-1], dt, mask, sdf, dx, dy, nu, U_inf, v_cycles=v_cycles,
                              fast_mode=fast_mode, brinkman_eta=brinkman_eta)
        states.append((u, v))
    acc = {"sdf": None if sdf is None else np.zeros_like(states[0][0]), "nu": 0.0, "U_inf": 0.0,
           "nu_abs": 0.0, "U_inf_abs": 0.0}
    for (u, v) in reversed(states):
        r = step_pure_vjp(u, v, dt, mask, sdf, dx, dy, nu, U_inf, gu, gv, None, v_cycles=v_cycles,
                          fast_mode=fast_mode, brinkman_eta=brinkman_eta)
        gu, gv = r["u"], r["v"]
        if sdf is not None:
            acc["sdf"] += r["sdf"]
        for key in ("nu", "U_inf", "nu_abs", "U_inf_abs"):
            acc[key] += r[key]
    acc["u"], acc["v"] = gu, gv
    return acc
