"""Known-answer checks of the oracle's new parts (converging multigrid, WENO5 on
the collocated and the staggered grid) and of the reference behaviours it
must reproduce (shape errors).  CPU only."""
import numpy as np
import pytest

from oracle import ref_np as R


def _direct_solve(b, dx, dy):
    """Sparse direct solve of the reference operator with the pinned outlet row."""
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    nx, ny = b.shape
    N = nx * ny
    rows, cols, vals = [], [], []
    for k in range(N):
        e = np.zeros(N)
        e[k] = 1.0
        col = R.lap_ref(e.reshape(nx, ny), dx, dy).ravel()
        nz = np.nonzero(col)[0]
        rows += list(nz)
        cols += [k] * len(nz)
        vals += list(col[nz])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(N, N)).tolil()
    for j in range(ny):
        r = (nx - 1) * ny + j
        A[r, :] = 0
        A[r, r] = 1.0
    bb = b.copy()
    bb[-1] = 0
    return spl.spsolve(A.tocsr(), bb.ravel()).reshape(nx, ny)


def test_converging_mg_matches_direct_solve():
    nx, ny, dx, dy = 64, 32, 1 / 64, 1 / 64
    b = np.random.default_rng(1).standard_normal((nx, ny))
    x = _direct_solve(b, dx, dy)
    p, info = R.mg_converge(b, dx, dy, rtol=1e-12, max_cycles=60)
    assert info["rel_residual"] <= 1e-12
    assert np.max(np.abs(p - x)) / np.max(np.abs(x)) < 1e-10


@pytest.mark.parametrize("shape", [(128, 32), (256, 64), (96, 48)])
def test_converging_mg_rate(shape):
    nx, ny = shape
    b = np.random.default_rng(2).standard_normal((nx, ny))
    p, info = R.mg_converge(b, 1 / 64, 1 / 64, rtol=1e-8, max_cycles=30)
    h = info["history"]
    rates = [h[i + 1] / h[i] for i in range(len(h) - 1)]
    assert info["rel_residual"] <= 1e-8
    assert max(rates) < 0.25          # a working multigrid, not a smoother


def test_warm_start_saves_cycles():
    nx, ny, dx = 128, 32, 1 / 64
    b = np.random.default_rng(3).standard_normal((nx, ny))
    p, info = R.mg_converge(b, dx, dx, rtol=1e-6)
    p2, info2 = R.mg_converge(b * 1.001, dx, dx, rtol=1e-6, p0=p)
    assert info2["cycles"] < info["cycles"]


@pytest.mark.parametrize("kind", ["smooth", "noise"])
def test_fp32_coarse_solve_changes_no_cycle(kind):
    """The GPU's exact separable coarse solve (cosine transforms and parallel
    cyclic reduction) runs in FP32.  Evaluated in FP32 (oracle restatement of
    the same schedule) or in FP64, it gives the converging multigrid the same
    cycle counts and the same contraction per cycle to 4 digits, down to a
    1e-10 relative residual, and the same converged pressure: the smooth
    modes the FP32 reduction resolves least accurately (the x-operator of the
    k = 0 cosine mode has condition ~4e5 at 512 cells) are corrected by the
    following cycles."""
    nx, ny, dx = 1024, 256, 1 / 64
    rng = np.random.default_rng(7)
    x = np.linspace(0, 1, nx)[:, None]
    y = np.linspace(0, 1, ny)[None, :]
    b = rng.standard_normal((nx, ny))
    if kind == "smooth":
        b = np.sin(3 * np.pi * x) * np.cos(2 * np.pi * y) + 0.1 * b
    p64, i64 = R.mg_converge(b, dx, dx, rtol=1e-10, max_cycles=30)
    p32, i32 = R.mg_converge(b, dx, dx, rtol=1e-10, max_cycles=30, coarse_dtype=np.float32)
    assert i64["direct_level"] > 0
    assert i32["cycles"] == i64["cycles"]
    h64, h32 = np.array(i64["history"]), np.array(i32["history"])
    assert np.max(np.abs(h32 / h64 - 1)) < 1e-3
    assert np.max(np.abs(p32 - p64)) <= 1e-8 * np.max(np.abs(p64))


def test_weno5_order():
    """Fifth-order convergence of the WENO5 derivative on a smooth field."""
    errs = []
    for n in (32, 64, 128):
        x = np.arange(n) / n * 2 * np.pi
        f = np.sin(x)[:, None] * np.ones((1, 4))
        d = R.weno5_derivative(f, np.ones_like(f), 2 * np.pi / n, 0, "wrap")
        errs.append(np.max(np.abs(d[:, 0] - np.cos(x))))
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(orders) > 4.5


def test_weno5_upwind_direction():
    n = 64
    x = np.arange(n) / n * 2 * np.pi
    f = np.sin(x)[:, None] * np.ones((1, 3))
    h = 2 * np.pi / n
    dpos = R.weno5_derivative(f, np.ones_like(f), h, 0, "wrap")
    dneg = R.weno5_derivative(f, -np.ones_like(f), h, 0, "wrap")
    assert np.max(np.abs(dpos - dneg)) < 1e-5       # both O(h^5)-consistent on smooth data
    assert not np.array_equal(dpos, dneg)           # but different stencils


@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_mac_weno5_order(sign):
    """Fifth-order convergence of the staggered WENO5 advection terms
    (mac_advection_terms, scheme='weno5') on smooth fields, both upwind
    directions.  The advecting velocity interpolated to the face
    (rk3_mac.py:239-253) is second order by itself, so the check isolates
    the derivatives: adv_u - (u du/dx + v_at_u du/dy) with exact
    derivatives, on faces at least four cells from every edge."""
    errs = []
    for n in (32, 64, 128):
        h = 2 * np.pi / n
        xf, xc = np.arange(n + 1) * h, (np.arange(n) + 0.5) * h
        U = lambda x, y: sign * (2.0 + np.sin(x) * np.cos(y))
        V = lambda x, y: sign * (1.5 + np.cos(x) * np.sin(y))
        uw = U(xf[:, None], xc[None, :])
        vw = V(xc[:, None], xf[None, :])
        au, av = R.mac_advection_terms(uw, vw, h, h, True, "weno5")
        vu, uv = R.v_to_u_face(vw), R.u_to_v_face(uw)
        xu, yu = xf[:, None], xc[None, :]
        xv, yv = xc[:, None], xf[None, :]
        ex_u = uw * sign * np.cos(xu) * np.cos(yu) - vu * sign * np.sin(xu) * np.sin(yu)
        ex_v = -uv * sign * np.sin(xv) * np.sin(yv) + vw * sign * np.cos(xv) * np.cos(yv)
        k = 4
        errs.append(max(np.max(np.abs(au - ex_u)[k:-k, k:-k]),
                        np.max(np.abs(av - ex_v)[k:-k, k:-k])))
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(orders) > 4.5, orders


def test_mac_upwind_scheme_unchanged():
    """scheme='upwind' of mac_advection_terms is the reference's blended
    upwind: a first-order scheme on the same smooth fields."""
    errs = []
    for n in (32, 64, 128):
        h = 2 * np.pi / n
        xf, xc = np.arange(n + 1) * h, (np.arange(n) + 0.5) * h
        uw = 2.0 + np.sin(xf[:, None]) * np.cos(xc[None, :])
        vw = 1.5 + np.cos(xc[:, None]) * np.sin(xf[None, :])
        au, _ = R.mac_advection_terms(uw, vw, h, h, True, "upwind")
        vu = R.v_to_u_face(vw)
        xu, yu = xf[:, None], xc[None, :]
        ex_u = uw * np.cos(xu) * np.cos(yu) - vu * np.sin(xu) * np.sin(yu)
        errs.append(np.max(np.abs(au - ex_u)[4:-4, 4:-4]))
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert 0.8 < min(orders) < 1.5, orders


@pytest.mark.parametrize("shape,ok", [((512, 96), True), ((64, 32), True), ((100, 64), False),
                                      ((64, 40), False), ((32, 16), False), ((2048, 512), True)])
def test_parity_level_rule(shape, ok):
    """multigrid_solver.py:96-106: non-divisible grids raise ValueError."""
    if ok:
        assert R.mg_levels_ok(*shape) == 4
    else:
        with pytest.raises(ValueError):
            R.mg_levels_ok(*shape)


def test_float32_oracle_close_to_float64():
    """The float32 evaluation (the timed CPU baseline) tracks float64."""
    rng = np.random.default_rng(4)
    nx, ny = 128, 32
    u = 1 + 0.01 * rng.standard_normal((nx, ny))
    v = 0.01 * rng.standard_normal((nx, ny))
    mask = np.ones((nx, ny))
    args = dict(dx=1 / 32, dy=1 / 32, nu=0.01, U_inf=1.0, brinkman_eta=1e-3, v_cycles=3)
    a = R.step_pure(u, v, 2e-3, mask, None, args["dx"], args["dy"], args["nu"], 1.0, v_cycles=3,
                    brinkman_eta=1e-3)
    b = R.step_pure(u.astype(np.float32), v.astype(np.float32), np.float32(2e-3),
                    mask.astype(np.float32), None, np.float32(args["dx"]), np.float32(args["dy"]),
                    np.float32(0.01), np.float32(1.0), v_cycles=3, brinkman_eta=np.float32(1e-3))
    for x, y in zip(a, b):
        assert y.dtype == np.float32
        assert np.max(np.abs(x - y)) / np.max(np.abs(x)) < 1e-4


def test_ensemble_draws_follow_the_workload():
    """The ensemble's instances: sizes from the four grids, diameter 8-32
    cells, centre at 10-20 % / 40-60 %, Re log-uniform in [100, 1000]."""
    from aerojax_gb300 import ensemble as E
    specs = E.draw_instances(256, seed=1)
    assert {(s.nx, s.ny) for s in specs} == set(E.SIZES)
    assert all(8 <= s.d_cells <= 32 and 0.1 <= s.cx_frac <= 0.2 and 0.4 <= s.cy_frac <= 0.6
               and 100 <= s.re <= 1000 for s in specs)
    logs = np.log([s.re for s in specs])
    assert abs(logs.mean() - 0.5 * (np.log(100) + np.log(1000))) < 0.15
