"""The oracle's reverse-mode step (oracle/adjoint_np.py), pinned by finite
differences of the pinned forward oracle.step_pure in FP64."""
import numpy as np
import pytest

from oracle import adjoint_np as A
from oracle import ref_np as R

NX, NY, DX, DT, NU, U = 64, 32, 0.05, 0.004, 0.02, 1.0


def _case(seed=0, sdf=True):
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid((np.arange(NX) + 0.5) * DX, (np.arange(NY) + 0.5) * DX, indexing="ij")
    s = R.sdf_cylinder(X, Y, 0.9, 0.8, 0.25)
    mask = R.mask_from_sdf(s, 0.5 * DX)
    u = U + 0.3 * rng.standard_normal((NX, NY))
    v = 0.3 * rng.standard_normal((NX, NY))
    return u, v, mask, (s if sdf else None), rng


def _loss(u, v, mask, sdf, nu, Uinf, gu, gv, gp, **kw):
    un, vn, p = R.step_pure(u, v, DT, mask, sdf, DX, DX, nu, Uinf, **kw)
    return float(np.sum(gu * un) + np.sum(gv * vn) + np.sum(gp * p))


def test_forward_stages_match_the_predictor():
    u, v, mask, sdf, _ = _case()
    for fast in (False, True):
        _, (un, vn), _, _ = A.forward_stages(u, v, DT, mask, sdf, DX, DX, NU, U, fast_mode=fast)
        un = np.where(mask > 0.5, un, 0.0)
        vn = np.where(mask > 0.5, vn, 0.0)
        un, vn = R.bc_collocated(un, vn, U)
        ru, rv = R.rk_step_unified(u, v, DT, NU, DX, DX, mask, sdf=sdf, U_inf=U, fast_mode=fast,
                                   brinkman_eta=0.005)
        assert np.allclose(un, ru, rtol=1e-12, atol=1e-12)
        assert np.allclose(vn, rv, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("cycles", [1, 3])
def test_multigrid_transpose(cycles):
    """<MG b, q> = <b, MG^T q> for the parity V-cycle (no early stop)."""
    rng = np.random.default_rng(4)
    b = rng.standard_normal((NX, NY))
    q = rng.standard_normal((NX, NY))
    ones = np.ones((NX, NY))
    p = R.poisson_multigrid(b, ones, DX, DX, 4, cycles, tolerance=0.0)
    bq = A.mg_vjp(q, DX, DX, 4, cycles)
    lhs, rhs = float(np.sum(p * q)), float(np.sum(b * bq))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


@pytest.mark.parametrize("fast,sdf,cycles", [(False, True, 1), (True, True, 1),
                                             (False, False, 1), (False, True, 2)])
def test_step_vjp_finite_differences(fast, sdf, cycles):
    u, v, mask, s, rng = _case(1, sdf)
    gu, gv, gp = (rng.standard_normal((NX, NY)) for _ in range(3))
    kw = dict(v_cycles=cycles, fast_mode=fast)
    r = A.step_pure_vjp(u, v, DT, mask, s, DX, DX, NU, U, gu, gv, gp, **kw)
    eps = 1e-6

    def fd(du=0.0, dv=0.0, ds=0.0, dnu=0.0, dU=0.0):
        lp = _loss(u + eps * du, v + eps * dv, mask, None if s is None else s + eps * ds,
                   NU + eps * dnu, U + eps * dU, gu, gv, gp, **kw)
        lm = _loss(u - eps * du, v - eps * dv, mask, None if s is None else s - eps * ds,
                   NU - eps * dnu, U - eps * dU, gu, gv, gp, **kw)
        return (lp - lm) / (2 * eps)

    du, dv = rng.standard_normal((NX, NY)), rng.standard_normal((NX, NY))
    checks = [(fd(du=du), float(np.sum(r["u"] * du))),
              (fd(dv=dv), float(np.sum(r["v"] * dv))),
              (fd(dnu=1.0), r["nu"]),
              (fd(dU=1.0), r["U_inf"])]
    if s is not None:
        ds = rng.standard_normal((NX, NY)) * DX
        checks.append((fd(ds=ds), float(np.sum(r["sdf"] * ds))))
    else:
        assert r["sdf"] is None
    for num, ana in checks:
        assert abs(num - ana) <= 1e-6 * max(abs(ana), 1e-3), (num, ana)
    assert r["cycles"] == cycles


def test_rollout_vjp_finite_differences():
    u, v, mask, s, rng = _case(2)
    gu, gv = rng.standard_normal((NX, NY)), rng.standard_normal((NX, NY))
    n = 3
    r = A.rollout_vjp(u, v, DT, mask, s, DX, DX, NU, U, n, gu, gv)
    du = rng.standard_normal((NX, NY))
    ds = rng.standard_normal((NX, NY)) * DX
    eps = 1e-6

    def loss(uu, ss, nu):
        (uf, vf), hist = A.rollout(uu, v, DT, mask, ss, DX, DX, nu, U, n)
        assert len(hist) == n
        return float(np.sum(gu * uf) + np.sum(gv * vf))

    num = (loss(u + eps * du, s, NU) - loss(u - eps * du, s, NU)) / (2 * eps)
    assert abs(num - np.sum(r["u"] * du)) <= 1e-6 * abs(num)
    num = (loss(u, s + eps * ds, NU) - loss(u, s - eps * ds, NU)) / (2 * eps)
    assert abs(num - np.sum(r["sdf"] * ds)) <= 1e-6 * abs(num)
    num = (loss(u, s, NU + eps) - loss(u, s, NU - eps)) / (2 * eps)
    assert abs(num - r["nu"]) <= 1e-6 * abs(num)


def _loss_gui(u, v, mask, sdf, nu, Uinf, gu, gv, gp, **kw):
    un, vn, p = R.step_gui(u, v, mask, DT, sdf=sdf, dx=DX, dy=DX, nu=nu, U_inf=Uinf,
                           mg=R.MGConfig(mode="parity", v_cycles=kw["v_cycles"]), **{
                               k: kw[k] for k in ("nu_hyper_ratio", "slip_walls", "fast_mode",
                                                   "brinkman_eta")})
    return float(np.sum(gu * un) + np.sum(gv * vn) + np.sum(gp * p))


@pytest.mark.parametrize("fast,hyper,slip,sdf,cycles", [
    (False, 0.0, True, True, 5), (False, 0.05, True, True, 2), (True, 0.05, False, True, 1),
    (False, 0.0, True, False, 3)])
def test_gui_step_vjp_finite_differences(fast, hyper, slip, sdf, cycles):
    """The collocated GUI step (BaselineSolver._step without LES): every
    cotangent against central differences of oracle.ref_np.step_gui."""
    u, v, mask, s, rng = _case(3, sdf)
    gu, gv, gp = (rng.standard_normal((NX, NY)) for _ in range(3))
    kw = dict(v_cycles=cycles, fast_mode=fast, nu_hyper_ratio=hyper, slip_walls=slip,
              brinkman_eta=1e-3)
    r = A.step_gui_vjp(u, v, DT, mask, s, DX, DX, NU, U, gu, gv, gp, **kw)
    eps = 1e-6

    def fd(du=0.0, dv=0.0, ds=0.0, dnu=0.0, dU=0.0):
        sp = None if s is None else s + eps * ds
        sm = None if s is None else s - eps * ds
        lp = _loss_gui(u + eps * du, v + eps * dv, mask, sp, NU + eps * dnu, U + eps * dU,
                       gu, gv, gp, **kw)
        lm = _loss_gui(u - eps * du, v - eps * dv, mask, sm, NU - eps * dnu, U - eps * dU,
                       gu, gv, gp, **kw)
        return (lp - lm) / (2 * eps)

    du, dv = rng.standard_normal((NX, NY)), rng.standard_normal((NX, NY))
    checks = [(fd(du=du), float(np.sum(r["u"] * du))),
              (fd(dv=dv), float(np.sum(r["v"] * dv))),
              (fd(dnu=1.0), r["nu"]),
              (fd(dU=1.0), r["U_inf"])]
    if s is not None:
        ds = rng.standard_normal((NX, NY)) * DX
        checks.append((fd(ds=ds), float(np.sum(r["sdf"] * ds))))
    for num, ana in checks:
        assert abs(num - ana) <= 1e-6 * max(abs(ana), 1e-3), (num, ana)
    un, vn, _ = r["out"]
    assert np.all(np.isfinite(un)) and np.all(np.isfinite(vn))
