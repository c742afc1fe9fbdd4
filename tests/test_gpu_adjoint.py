"""aj_step_vjp (reverse mode of step_pure) on the GPU against the FP64 oracle
(oracle/adjoint_np.py, itself pinned by finite differences), through the
C ABI; linearity and determinism at 2048x512; the rollout's reverse scan."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DX, DT, NU, U = 0.05, 0.004, 0.02, 1.0


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _case(nx, ny, seed, dx=DX):
    from oracle import ref_np as R
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx, indexing="ij")
    s = R.sdf_cylinder(X, Y, 0.28 * nx * dx, 0.5 * ny * dx, 0.08 * ny * dx)
    mask = R.mask_from_sdf(s, 0.5 * dx)
    u = U + 0.3 * rng.standard_normal((nx, ny))
    v = 0.3 * rng.standard_normal((nx, ny))
    f32 = lambda a: np.asarray(a, np.float32)
    return f32(u), f32(v), f32(mask), f32(s), rng


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _t(a, dev):
    return torch.as_tensor(np.asarray(a, np.float32), device=dev)


def _scalar_ok(got, ref, key, rel):
    """d/d nu and d/d U_inf are sums of many terms that largely cancel (for
    d/d nu on random fields |sum| can be 1e-5 of sum |terms|): the FP32
    error is bounded against the oracle's magnitude scale of the sum, or
    ``rel`` of the value, whichever is larger."""
    tol = max(rel * abs(ref[key]), 1e-7 * ref[key + "_abs"])
    return abs(got - ref[key]) <= tol


@pytest.mark.parametrize("fast,use_sdf,cycles", [(False, True, 1), (True, True, 1),
                                                 (False, False, 1), (False, True, 3)])
def test_step_vjp_matches_oracle(dev, fast, use_sdf, cycles):
    """Every cotangent within 1e-4 (relative L2; FP32 reverse pass against
    FP64) of the oracle's on a 128x64 cylinder case."""
    from oracle import adjoint_np as A
    from aerojax_gb300 import adjoint as ADJ
    from aerojax_gb300.params import SimState
    nx, ny = 128, 64
    u, v, mask, s, rng = _case(nx, ny, 11)
    sdf = s if use_sdf else None
    gu, gv, gp = (rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(3))
    ref = A.step_pure_vjp(u, v, DT, mask, sdf, DX, DX, NU, U, gu, gv, gp, v_cycles=cycles,
                          fast_mode=fast)
    st = SimState(u=_t(u, dev), v=_t(v, dev), p=None, u_prev=None, v_prev=None, c=None, dt=DT,
                  iteration=0)
    got = ADJ.step_pure_vjp(st, _t(mask, dev), None if sdf is None else _t(sdf, dev), DX, DX, NU,
                            U, _t(gu, dev), _t(gv, dev), _t(gp, dev), v_cycles=cycles,
                            fast_mode=fast)
    assert _rel(got["u"].cpu(), ref["u"]) <= 1e-4
    assert _rel(got["v"].cpu(), ref["v"]) <= 1e-4
    if use_sdf:
        assert _rel(got["sdf"].cpu(), ref["sdf"]) <= 1e-4
    else:
        assert got["sdf"] is None and ref["sdf"] is None
    assert _scalar_ok(got["nu"], ref, "nu", 1e-4), (got["nu"], ref["nu"], ref["nu_abs"])
    assert _scalar_ok(got["U_inf"], ref, "U_inf", 1e-4), (got["U_inf"], ref["U_inf"])


def test_step_vjp_full_size(dev):
    """2048x512: against the oracle, linear in the cotangent, and bit-for-bit
    repeatable."""
    from oracle import adjoint_np as A
    from aerojax_gb300.adjoint import StepVjp, _config
    nx, ny, dx = 2048, 512, 1.0 / 128
    u, v, mask, s, rng = _case(nx, ny, 12, dx)
    dt = 2e-4
    cfg = _config(nx, ny, dx, dx, 1e-3, U, dt, True)
    op = StepVjp(cfg, dev)
    M, S = _t(mask, dev), _t(s, dev)
    op.prepare(M, S)
    ud, vd = _t(u, dev), _t(v, dev)
    g1 = [rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(3)]
    g2 = [rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(3)]

    def run(g):
        op.zero_grad()
        gu, gv = op(ud, vd, M, *(_t(x, dev) for x in g))
        return gu.cpu().numpy().copy(), gv.cpu().numpy().copy(), op.gsdf.cpu().numpy().copy(), \
            op.gscal.cpu().numpy().copy()

    r1 = run(g1)
    r1b = run(g1)
    for a, b in zip(r1, r1b):
        assert np.array_equal(a, b)                   # deterministic
    r2 = run(g2)
    r12 = run([2.0 * a - 0.5 * b for a, b in zip(g1, g2)])
    for a, b, c in zip(r1[:3], r2[:3], r12[:3]):
        assert _rel(c, 2.0 * a - 0.5 * b) <= 1e-5
    ref = A.step_pure_vjp(u, v, dt, mask, s, dx, dx, 1e-3, U, *g1)
    assert _rel(r1[0], ref["u"]) <= 1e-4
    assert _rel(r1[1], ref["v"]) <= 1e-4
    assert _rel(r1[2], ref["sdf"]) <= 1e-4
    assert _scalar_ok(r1[3][0], ref, "nu", 1e-4), (r1[3][0], ref["nu"], ref["nu_abs"])
    assert _scalar_ok(r1[3][1], ref, "U_inf", 1e-4), (r1[3][1], ref["U_inf"])


def test_rollout_vjp_matches_oracle(dev):
    """Four steps forward (history kept on the device) and the reverse scan:
    the initial state's, the SDF's and nu's cotangents match the oracle's."""
    from oracle import adjoint_np as A
    from aerojax_gb300 import adjoint as ADJ
    from aerojax_gb300.params import SimState
    nx, ny, n = 128, 64, 4
    u, v, mask, s, rng = _case(nx, ny, 13)
    gu, gv = (rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(2))
    params = {"dx": DX, "dy": DX, "nu": NU, "U_inf": U, "sdf": _t(s, dev)}
    st = SimState(u=_t(u, dev), v=_t(v, dev), p=None, u_prev=None, v_prev=None, c=None, dt=DT,
                  iteration=0)
    final, hist = ADJ.differentiable_rollout(st, _t(mask, dev), params, n)
    assert hist[0].shape == (n, nx, ny) and final.iteration == n
    (ru, rv), _ = A.rollout(u, v, DT, mask, s, DX, DX, NU, U, n)
    assert _rel(final.u.cpu(), ru) <= 1e-5
    got = ADJ.rollout_vjp(st, _t(mask, dev), params, n, _t(gu, dev), _t(gv, dev), history=hist)
    ref = A.rollout_vjp(u, v, DT, mask, s, DX, DX, NU, U, n, gu, gv)
    assert _rel(got["u"].cpu(), ref["u"]) <= 2e-4
    assert _rel(got["v"].cpu(), ref["v"]) <= 2e-4
    assert _rel(got["sdf"].cpu(), ref["sdf"]) <= 2e-4
    assert _scalar_ok(got["nu"], ref, "nu", 2e-4), (got["nu"], ref["nu"], ref["nu_abs"])
    assert _scalar_ok(got["U_inf"], ref, "U_inf", 2e-4), (got["U_inf"], ref["U_inf"])


@pytest.mark.parametrize("fast,hyper,slip,use_sdf,cycles", [
    (False, 0.05, True, True, 2), (True, 0.0, False, True, 1), (False, 0.05, False, False, 5)])
def test_gui_step_vjp_matches_oracle(dev, fast, hyper, slip, use_sdf, cycles):
    """The collocated GUI step without LES (hyperviscosity, both wall
    conditions): every cotangent within 1e-4 of the oracle's at 128x64."""
    from oracle import adjoint_np as A
    from aerojax_gb300 import adjoint as ADJ
    nx, ny = 128, 64
    u, v, mask, s, rng = _case(nx, ny, 14)
    sdf = s if use_sdf else None
    gu, gv, gp = (rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(3))
    kw = dict(v_cycles=cycles, fast_mode=fast, nu_hyper_ratio=hyper, slip_walls=slip,
              brinkman_eta=1e-3)
    ref = A.step_gui_vjp(u, v, DT, mask, sdf, DX, DX, NU, U, gu, gv, gp, **kw)
    got = ADJ.gui_step_vjp(_t(u, dev), _t(v, dev), _t(mask, dev), DT, _t(gu, dev), _t(gv, dev),
                           _t(gp, dev), sdf=None if sdf is None else _t(sdf, dev), dx=DX, dy=DX,
                           nu=NU, U_inf=U, nu_hyper_ratio=hyper, slip_walls=slip,
                           fast_mode=fast, brinkman_eta=1e-3, multigrid_v_cycles=cycles)
    assert _rel(got["u"].cpu(), ref["u"]) <= 1e-4
    assert _rel(got["v"].cpu(), ref["v"]) <= 1e-4
    if use_sdf:
        assert _rel(got["sdf"].cpu(), ref["sdf"]) <= 1e-4
    assert _scalar_ok(got["nu"], ref, "nu", 1e-4), (got["nu"], ref["nu"], ref["nu_abs"])
    assert _scalar_ok(got["U_inf"], ref, "U_inf", 1e-4), (got["U_inf"], ref["U_inf"])


def test_ragged_grid_parity_solve_and_reverse_mode(dev):
    """96x80 (partial tiles on every level, a 6x5 coarsest level): the parity
    multigrid (collocated and MAC) against the oracle's V-cycle, and the
    reverse-mode step against the oracle's."""
    import aerojax_gb300 as aj
    from oracle import adjoint_np as A
    from oracle import ref_np as R
    from aerojax_gb300 import adjoint as ADJ
    from aerojax_gb300.params import SimState
    nx, ny = 96, 80
    u, v, mask, s, rng = _case(nx, ny, 15)
    b = rng.standard_normal((nx, ny)).astype(np.float32)
    for mac in (False, True):
        solve = aj.poisson_multigrid_mac if mac else aj.poisson_multigrid
        p = solve(_t(b, dev), _t(mask, dev), DX, DX, v_cycles=3)
        ref = R.poisson_multigrid(b.astype(np.float64), mask.astype(np.float64), DX, DX, 4, 3,
                                  mac=mac)
        err = float(np.max(np.abs(p.cpu().numpy() - ref)) / np.max(np.abs(ref)))
        assert err < 1e-5, (mac, err)
    gu, gv, gp = (rng.standard_normal((nx, ny)).astype(np.float32) for _ in range(3))
    ref = A.step_pure_vjp(u, v, DT, mask, s, DX, DX, NU, U, gu, gv, gp, v_cycles=2)
    st = SimState(u=_t(u, dev), v=_t(v, dev), p=None, u_prev=None, v_prev=None, c=None, dt=DT,
                  iteration=0)
    got = ADJ.step_pure_vjp(st, _t(mask, dev), _t(s, dev), DX, DX, NU, U, _t(gu, dev),
                            _t(gv, dev), _t(gp, dev), v_cycles=2)
    for name in ("u", "v", "sdf"):
        assert _rel(got[name].cpu(), ref[name]) <= 1e-4, name
