"""GPU parity of the WENO5 advection against the float64 oracle.

WENO5-JS has no reference counterpart (the reference plumbs ``weno_epsilon``
through ``solver/pure_functions/step.py:52`` but advects with first-order
upwind, ``advection_schemes/rk3_simple_new.py:287-298``); the oracle's
``weno5_derivative`` restates Jiang & Shu (1996) and is pinned by its
convergence order (``tests/test_oracle_properties.py``).  Here the CUDA stage
kernels are compared with that oracle through the C ABI:

* the collocated predictor (``rk_step_unified`` with ``advection='weno5'``):
  RK3 and RK2, with and without hyperviscosity, slip and no-slip walls, an
  SDF-driven chi, the periodic (Taylor-Green) padding, on ragged grids;
* the MAC predictor (``rk_step_unified_mac`` with ``advection='weno5'``);
* the 512x96 cylinder workload with WENO5 over 200 steps (step_pure, parity
  multigrid with 3 V-cycles, CFL 0.5), every GPU step against the oracle step
  taken from the same (GPU) input state.

Tolerance: max|gpu - ref| / max|ref| <= 1e-5 on u, v (and p)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = a.detach().double().cpu().numpy() if hasattr(a, "detach") else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def T(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device="cuda")


def H(t):
    return t.detach().double().cpu().numpy()


def _fields(nx, ny, seed, mac=False):
    """Smooth vortical velocity plus noise, rounded to FP32 (the GPU's input)."""
    rng = np.random.default_rng(seed)
    nxu, nyu = (nx + 1, ny) if mac else (nx, ny)
    nxv, nyv = (nx, ny + 1) if mac else (nx, ny)
    xu = np.linspace(0, 1, nxu)[:, None]
    yu = np.linspace(0, 1, nyu)[None, :]
    xv = np.linspace(0, 1, nxv)[:, None]
    yv = np.linspace(0, 1, nyv)[None, :]
    u = 1.0 + 0.3 * np.sin(2 * np.pi * xu) * np.cos(3 * np.pi * yu) \
        + 0.05 * rng.standard_normal((nxu, nyu))
    v = 0.3 * np.cos(4 * np.pi * xv) * np.sin(2 * np.pi * yv) \
        - 0.1 + 0.05 * rng.standard_normal((nxv, nyv))
    f = np.float32
    return u.astype(f).astype(np.float64), v.astype(f).astype(np.float64)


def _cylinder(nx, ny, dx, dy, cells=8.0):
    from oracle import ref_np as R
    X, Y = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dy, indexing="ij")
    sdf = R.sdf_cylinder(X, Y, 0.3 * nx * dx, 0.5 * ny * dy, cells * dx)
    mask = R.mask_from_sdf(sdf, 0.5 * dx)
    f = np.float32
    return sdf.astype(f).astype(np.float64), mask.astype(f).astype(np.float64)


@pytest.mark.parametrize("shape,fast,hyper,slip,flow,use_sdf", [
    ((100, 70), False, 0.0, True, "von_karman", True),
    ((100, 70), True, 0.0, True, "von_karman", True),
    ((96, 80), False, 0.05, True, "von_karman", True),
    ((96, 80), True, 0.05, False, "von_karman", False),
    ((97, 61), False, 0.0, False, "von_karman", False),
    ((64, 48), False, 0.02, True, "taylor_green", False),
])
def test_weno5_predictor_collocated(cuda_lib, shape, fast, hyper, slip, flow, use_sdf):
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    nx, ny = shape
    dx, dy, dt, nu = 1 / 64, 1 / 48, 2e-3, 4e-3
    u, v = _fields(nx, ny, nx * 7 + ny)
    sdf, mask = _cylinder(nx, ny, dx, dy)
    if not use_sdf:
        sdf = None
    kw = dict(U_inf=1.0, nu_hyper_ratio=hyper, slip_walls=slip, fast_mode=fast,
              brinkman_eta=1e-3, flow_type=flow)
    ur, vr = R.rk_step_unified(u, v, dt, nu, dx, dy, mask, sdf=sdf, advection="weno5", **kw)
    ug, vg = aj.rk_step_unified(T(u), T(v), dt, nu, dx, dy, T(mask),
                                sdf=None if sdf is None else T(sdf), advection="weno5", **kw)
    assert rel(ug, ur) < TOL
    assert rel(vg, vr) < TOL
    # the WENO5 flux must differ from the upwind one on these fields (the
    # kernel really took the WENO5 path)
    uu, _ = R.rk_step_unified(u, v, dt, nu, dx, dy, mask, sdf=sdf, advection="upwind", **kw)
    assert rel(uu, ur) > 100 * TOL


def test_weno5_predictor_with_eddy_viscosity(cuda_lib):
    """WENO5 with a cell field of eddy viscosity, passed the way the GUI
    collocated step passes it (nu + nu_sgs as nu and nu_sgs again,
    step_handlers.py:76,84-85)."""
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    nx, ny, dx, dy, dt, nu = 128, 48, 1 / 64, 1 / 64, 2e-3, 2e-3
    u, v = _fields(nx, ny, 3)
    sdf, mask = _cylinder(nx, ny, dx, dy)
    nsg = R.constant_smagorinsky(u, v, dx, dy, dx, 0.17).astype(np.float32).astype(np.float64)
    ur, vr = R.rk_step_unified(u, v, dt, nu + nsg, dx, dy, mask, sdf=sdf, nu_sgs=nsg,
                               brinkman_eta=1e-3, advection="weno5")
    ug, vg = aj.rk_step_unified(T(u), T(v), dt, nu, dx, dy, T(mask), sdf=T(sdf), nu_sgs=T(nsg),
                                brinkman_eta=1e-3, double_count=True, advection="weno5")
    assert rel(ug, ur) < TOL
    assert rel(vg, vr) < TOL


@pytest.mark.parametrize("shape,fast,hyper,slip", [
    ((96, 64), False, 0.0, True),
    ((96, 64), True, 0.05, True),
    ((100, 70), False, 0.02, False),
    ((67, 45), True, 0.0, False),
])
def test_weno5_predictor_mac(cuda_lib, shape, fast, hyper, slip):
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    nx, ny = shape
    dx, dy, dt, nu = 1 / 64, 1 / 48, 2e-3, 4e-3
    u, v = _fields(nx, ny, nx + 3 * ny, mac=True)
    _, mask = _cylinder(nx, ny, dx, dy)
    nsg = R.constant_smagorinsky(*R.interpolate_to_cell_center(u, v), dx, dy, dx, 0.17)
    nsg = nsg.astype(np.float32).astype(np.float64)
    kw = dict(U_inf=1.0, nu_hyper_ratio=hyper, slip_walls=slip, fast_mode=fast,
              brinkman_eta=1e-3)
    ur, vr = R.rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, nu_sgs=nsg, advection="weno5", **kw)
    ug, vg = aj.rk_step_unified_mac(T(u), T(v), dt, nu, dx, dy, T(mask), nu_sgs=T(nsg),
                                    advection="weno5", **kw)
    assert rel(ug, ur) < TOL
    assert rel(vg, vr) < TOL
    ub, _ = R.rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, nu_sgs=nsg, **kw)
    assert rel(ub, ur) > 100 * TOL


def test_cylinder_512x96_weno5_200_steps(cuda_lib):
    """The 512x96 cylinder workload as specified: WENO5, RK3, 3 parity
    V-cycles, dt from CFL 0.5 on the device, 200 steps.  Each GPU step is
    compared with the oracle step from the same input state."""
    import aerojax_gb300 as aj
    from aerojax_gb300 import configs
    from oracle import ref_np as R
    case = configs.cylinder_512x96(advection="weno5")
    c = case["cfg"]
    assert c.advection_scheme == "weno5"
    mask, sdf = case["mask"], case["sdf"]
    plan = aj.get_plan(c, mask.device)
    plan.prepare(mask, sdf)
    mh, sh = H(mask), H(sdf)
    u, v = case["u"], case["v"]
    worst = [0.0, 0.0, 0.0]
    for step in range(200):
        un, vn, p = aj.run_step(plan, u, v, mask)
        dt = plan.stats()["dt"]
        uh, vh = H(u), H(v)
        dt_ref = R.compute_cfl_timestep(uh.astype(np.float32), vh.astype(np.float32), c.dx, c.dy,
                                        c.nu, 0.5, 1e-6, 1.0)
        assert dt == pytest.approx(dt_ref, rel=1e-6), step
        ur, vr, pr = R.step_pure(uh, vh, dt, mh, sh, c.dx, c.dy, c.nu, c.U_inf, v_cycles=3,
                                 brinkman_eta=c.brinkman_eta, advection="weno5")
        e = (rel(un, ur), rel(vn, vr), rel(p, pr))
        worst = [max(a, b) for a, b in zip(worst, e)]
        assert e[0] < TOL and e[1] < TOL and e[2] < TOL, (step, e)
        u, v = un, vn
    print("worst relative error over 200 WENO5 steps (u, v, p):", worst)
    assert float(v.abs().max()) > 1e-3      # the wake has started to move
