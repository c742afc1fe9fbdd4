"""GPU parity: every golden fixture (the reference's own source run in float64)
reproduced by the CUDA path through the C ABI, in FP32.

Tolerance: max|gpu - ref| / max|ref| <= 1e-5 for velocity and pressure
(the FP32 bar).  The one exception is the dynamic Smagorinsky model, whose
bound is the distance of the reference's own algorithm evaluated in FP32 from
its FP64 run (test_les)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel(a, b):
    a = a.detach().double().cpu().numpy() if hasattr(a, "detach") else np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def T(x):
    import torch
    return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device="cuda")


@pytest.mark.parametrize("name", ["mg_64x32", "mg_128x48"])
def test_multigrid_parity(cuda_lib, name):
    import aerojax_gb300 as aj
    g = golden(name)
    p = aj.poisson_multigrid(T(g["rhs"]), T(g["mask"]), float(g["dx"]), float(g["dy"]),
                             v_cycles=int(g["v_cycles"]))
    pm = aj.poisson_multigrid_mac(T(g["rhs"]), T(g["mask"]), float(g["dx"]), float(g["dy"]),
                                  v_cycles=int(g["v_cycles"]))
    assert rel(p, g["p"]) < TOL
    assert rel(pm, g["p_mac"]) < TOL


@pytest.mark.parametrize("name", ["rk3", "rk2", "rk3_hyper", "rk3_field"])
def test_predictor_collocated(cuda_lib, name):
    import aerojax_gb300 as aj
    g = golden("pred_" + name)
    field = g["nu_sgs"].shape != (1, 1)
    us, vs = aj.rk_step_unified(T(g["u"]), T(g["v"]), float(g["dt"]), 0.01 if field else float(g["nu"]),
                                float(g["dx"]), float(g["dy"]), T(g["mask"]), sdf=T(g["sdf"]),
                                U_inf=float(g["U"]), nu_sgs=T(g["nu_sgs"]) if field else None,
                                nu_hyper_ratio=float(g["hyper"]), fast_mode=bool(g["fast"]),
                                brinkman_eta=float(g["eta"]), double_count=field)
    assert rel(us, g["u_star"]) < TOL
    assert rel(vs, g["v_star"]) < TOL


@pytest.mark.parametrize("name", ["mac_rk3", "mac_rk2_les_hyper"])
def test_predictor_mac(cuda_lib, name):
    import aerojax_gb300 as aj
    g = golden("pred_" + name)
    field = g["nu_sgs"].shape != (1, 1)
    us, vs = aj.rk_step_unified_mac(T(g["u"]), T(g["v"]), float(g["dt"]), float(g["nu"]),
                                    float(g["dx"]), float(g["dy"]), T(g["mask"]), U_inf=float(g["U"]),
                                    nu_sgs=T(g["nu_sgs"]) if field else None,
                                    nu_hyper_ratio=float(g["hyper"]), fast_mode=bool(g["fast"]),
                                    brinkman_eta=float(g["eta"]))
    assert rel(us, g["u_star"]) < TOL
    assert rel(vs, g["v_star"]) < TOL


@pytest.mark.parametrize("shape,slip,les", [((100, 68), True, True), ((70, 44), False, True),
                                             ((34, 8), True, False), ((256, 64), True, True)])
def test_predictor_mac_tile(cuda_lib, shape, slip, les):
    """The MAC RK3 predictor on grids the one-kernel tile path covers (nx
    even, ny a multiple of 4), whole and partial 32x32 tiles, slip and
    no-slip walls, with and without eddy viscosity, against the oracle."""
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    nx, ny = shape
    rng = np.random.default_rng(nx * ny)
    dx, dy, dt, nu, eta = 1 / 64, 1 / 48, 2e-3, 4e-3, 1e-3
    u = (1 + 0.1 * rng.standard_normal((nx + 1, ny))).astype(np.float32).astype(np.float64)
    v = (0.1 * rng.standard_normal((nx, ny + 1))).astype(np.float32).astype(np.float64)
    X, Y = np.meshgrid((np.arange(nx) + .5) * dx, (np.arange(ny) + .5) * dy, indexing="ij")
    mask = R.mask_from_sdf(R.sdf_cylinder(X, Y, 0.4 * nx * dx, 0.5 * ny * dy, 3 * dx), 0.5 * dx)
    mask = mask.astype(np.float32).astype(np.float64)
    nsg = (1e-3 * rng.random((nx, ny))).astype(np.float32).astype(np.float64) if les else None
    ur, vr = R.rk_step_unified_mac(u, v, dt, nu, dx, dy, mask, nu_sgs=nsg, slip_walls=slip,
                                   brinkman_eta=eta)
    ug, vg = aj.rk_step_unified_mac(T(u), T(v), dt, nu, dx, dy, T(mask),
                                    nu_sgs=T(nsg) if les else None, slip_walls=slip,
                                    brinkman_eta=eta)
    assert rel(ug, ur) < TOL
    assert rel(vg, vr) < TOL


def test_les(cuda_lib):
    import aerojax_gb300 as aj
    g = golden("les")
    c = aj.constant_smagorinsky(T(g["u"]), T(g["v"]), float(g["dx"]), float(g["dy"]),
                                float(g["delta"]), 0.17)
    d, cd = aj.dynamic_smagorinsky(T(g["u"]), T(g["v"]), float(g["dx"]), float(g["dy"]),
                                   float(g["delta"]))
    assert rel(c, g["nu_const"]) < TOL
    # C_d = <LM>/(<MM>+1e-8): L_ij = filter(u_i)filter(u_j) - filter(u_i u_j)
    # cancels to ~1e-4 of its terms, so the reference's own algorithm
    # evaluated in FP32 departs from its FP64 run by ~1.2e-4 on this field.
    # The GPU must be no further from FP64 than that FP32 evaluation.
    d32, cd32 = _dynamic_fp32(g)
    assert rel(cd, g["cd"]) <= max(TOL, 2.0 * rel(cd32, g["cd"]))
    assert rel(d, g["nu_dyn"]) <= max(TOL, 2.0 * rel(d32, g["nu_dyn"]))
    assert rel(d32, g["nu_dyn"]) > 10 * TOL     # the bound is the FP32 evaluation's, not 1e-5


def _dynamic_fp32(g):
    """The oracle's dynamic Smagorinsky in FP32 arithmetic (the reference's
    default precision, solver/config.py:28) on the fixture's inputs."""
    from oracle import ref_np as R
    f = np.float32
    return R.dynamic_smagorinsky(g["u"].astype(f), g["v"].astype(f), f(g["dx"]), f(g["dy"]),
                                 f(g["delta"]))


def test_step_pure(cuda_lib):
    import aerojax_gb300 as aj
    g = golden("step_pure")
    st = aj.SimState(u=T(g["u"]), v=T(g["v"]), p=None, u_prev=None, v_prev=None, c=None,
                     dt=float(g["dt"]), iteration=0)
    out = aj.step_pure(st, T(g["mask"]), T(g["sdf"]), float(g["dx"]), float(g["dy"]), float(g["nu"]),
                       float(g["U"]), v_cycles=int(g["v_cycles"]), brinkman_eta=float(g["eta"]))
    assert out.iteration == 1
    assert rel(out.u, g["u_new"]) < TOL
    assert rel(out.v, g["v_new"]) < TOL
    assert rel(out.p, g["p"]) < TOL


@pytest.mark.parametrize("name", ["gui_col_les", "gui_col_dyn", "gui_col_plain", "gui_mac_les",
                                  "gui_mac_plain"])
def test_step_gui(cuda_lib, name):
    import aerojax_gb300 as aj
    g = golden("step_" + name)
    mac = "mac" in name
    nx, ny = g["mask"].shape
    h = aj.StepHandler(nx, ny, float(g["dx"]), float(g["dy"]), float(g["nu"]), float(g["U"]),
                       grid_type="mac" if mac else "collocated", use_les=bool(g["use_les"]),
                       les_model="dynamic_smagorinsky" if int(g["dynamic"]) else "smagorinsky",
                       smagorinsky_constant=float(g["cs"]), nu_hyper_ratio=float(g["hyper"]),
                       brinkman_eta=float(g["eta"]), multigrid_v_cycles=int(g["v_cycles"]),
                       sdf=None if mac else T(g["sdf"]), dt=float(g["dt"]))
    u, v, p = h._step(T(g["u"]), T(g["v"]), T(g["mask"]))
    if int(g["dynamic"]):
        # dynamic C_d (see test_les): bounded by the reference's own step
        # evaluated in FP32 from the same inputs
        from oracle import ref_np as R
        f = np.float32
        r32 = R.step_gui(g["u"].astype(f), g["v"].astype(f), g["mask"].astype(f), f(g["dt"]),
                         sdf=None if mac else g["sdf"].astype(f), dx=f(g["dx"]), dy=f(g["dy"]),
                         nu=f(g["nu"]), U_inf=f(g["U"]), grid_type="mac" if mac else "collocated",
                         use_les=True, les_model="dynamic_smagorinsky",
                         smagorinsky_constant=f(g["cs"]), nu_hyper_ratio=f(g["hyper"]),
                         brinkman_eta=f(g["eta"]), v_cycles=int(g["v_cycles"]))
        for got, key, ref32 in ((u, "u_new", r32[0]), (v, "v_new", r32[1]), (p, "p", r32[2])):
            assert rel(got, g[key]) <= max(TOL, 2.0 * rel(ref32, g[key])), key
        return
    assert rel(u, g["u_new"]) < TOL
    assert rel(v, g["v_new"]) < TOL
    assert rel(p, g["p"]) < TOL


def test_cfl(cuda_lib):
    import aerojax_gb300 as aj
    g = golden("cfl")
    a = aj.compute_cfl_timestep(T(g["u"]), T(g["v"]), float(g["dx"]), float(g["dy"]), float(g["nu"]),
                                cfl_target=0.5, dt_min=1e-5, dt_max=0.05)
    b = aj.compute_cfl_timestep(T(g["um"]), T(g["vm"]), float(g["dx"]), float(g["dy"]),
                                float(g["nu"]), cfl_target=0.5, dt_min=1e-5, dt_max=0.05)
    assert float(a.item()) == pytest.approx(float(g["dt"]), rel=1e-6)
    assert float(b.item()) == pytest.approx(float(g["dt_mac"]), rel=1e-6)


def test_geometry(cuda_lib):
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    g = golden("geometry")
    nx, ny = g["X"].shape
    lx, ly = float(g["X"][-1, 0]), float(g["Y"][0, -1])
    eps = 0.05 * lx / nx
    for kind, geo, key in [("naca4", (1.5, 10.0, 1.5, 1.5, 0.0, 0.0, 0.12), "sdf_naca0012"),
                           ("naca4", (1.5, 5.0, 1.5, 1.5, 0.02, 0.4, 0.12), "sdf_naca2412"),
                           ("cyl3_row", (2.0, 1.5, 0.5, 0.8), "sdf_three")]:
        mask, sdf = aj.make_geometry(kind, nx, ny, lx, ly, geo, eps)
        ref = g[key]
        assert np.nanmax(np.abs(sdf.cpu().numpy() - ref)) < 1e-6
        mref = R.mask_from_sdf(ref, eps)
        assert np.max(np.abs(mask.cpu().numpy() - mref)) < 1e-5
    # the triangle of three cylinders has no reference counterpart: the oracle's
    # SDF (sdf_three_cylinders_triangle) on the fixture's grid
    X, Y = g["X"], g["Y"]
    geo = (2.0, 1.5, 0.5, 0.8)
    mask, sdf = aj.make_geometry("cyl3_tri", nx, ny, lx, ly, geo, eps)
    ref = R.sdf_three_cylinders_triangle(X, Y, *geo)
    assert np.max(np.abs(sdf.cpu().numpy() - ref)) < 1e-6
    assert np.max(np.abs(mask.cpu().numpy() - R.mask_from_sdf(ref, eps))) < 1e-5


def test_shape_error_like_reference(cuda_lib):
    import aerojax_gb300 as aj
    import torch
    rhs = torch.zeros((100, 64), device="cuda")
    with pytest.raises(ValueError):
        aj.poisson_multigrid(rhs, torch.ones_like(rhs), 0.01, 0.01)


def test_step_gui_no_slip_walls_against_oracle(cuda_lib):
    """The collocated GUI step with no-slip walls (slip_walls=False) and
    hyperviscosity, which the golden fixtures (slip walls) do not cover,
    against the oracle's step_gui on a 96x80 cylinder case."""
    import aerojax_gb300 as aj
    from oracle import ref_np as R
    nx, ny, dx, dt = 96, 80, 0.05, 0.004
    rng = np.random.default_rng(21)
    X, Y = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx, indexing="ij")
    sdf = R.sdf_cylinder(X, Y, 1.4, 2.0, 0.4)
    mask = R.mask_from_sdf(sdf, 0.5 * dx)
    u = 1.0 + 0.1 * rng.standard_normal((nx, ny))
    v = 0.1 * rng.standard_normal((nx, ny))
    kw = dict(nu_hyper_ratio=0.05, slip_walls=False, brinkman_eta=1e-3)
    ur, vr, pr = R.step_gui(u, v, mask, dt, sdf=sdf, dx=dx, dy=dx, nu=0.02, U_inf=1.0,
                            v_cycles=3, **kw)
    h = aj.StepHandler(nx, ny, dx, dx, 0.02, 1.0, grid_type="collocated", use_les=False,
                       multigrid_v_cycles=3, sdf=T(sdf), dt=dt, **kw)
    ug, vg, pg = h._step(T(u), T(v), T(mask))
    assert rel(ug, ur) < TOL
    assert rel(vg, vr) < TOL
    assert rel(pg, pr) < TOL


@pytest.mark.parametrize("tag", ["ldc", "tg"])
def test_other_flow_types(cuda_lib, tag):
    """Lid-driven cavity and Taylor-Green through the C ABI against the
    reference's own results (fixtures flow_*): the parity multigrid on both
    grids (mean subtraction and centre pin; the wrapped residual), step_pure,
    and the GUI step on the collocated and the MAC grid."""
    import aerojax_gb300 as aj
    g = golden(f"flow_mg_{tag}")
    flow = str(g["flow"])
    p = aj.poisson_multigrid(T(g["rhs"]), T(g["mask"]), float(g["dx"]), float(g["dy"]),
                             v_cycles=int(g["v_cycles"]), flow_type=flow)
    pm = aj.poisson_multigrid_mac(T(g["rhs"]), T(g["mask"]), float(g["dx"]), float(g["dy"]),
                                  v_cycles=int(g["v_cycles"]), flow_type=flow)
    assert rel(p, g["p"]) < TOL, rel(p, g["p"])
    assert rel(pm, g["p_mac"]) < TOL, rel(pm, g["p_mac"])
    g = golden(f"flow_step_pure_{tag}")
    st = aj.SimState(u=T(g["u"]), v=T(g["v"]), p=None, u_prev=None, v_prev=None, c=None,
                     dt=float(g["dt"]), iteration=0)
    out = aj.step_pure(st, T(g["mask"]), T(g["sdf"]), float(g["dx"]), float(g["dy"]),
                       float(g["nu"]), float(g["U"]), v_cycles=int(g["v_cycles"]),
                       brinkman_eta=float(g["eta"]), flow_type=flow)
    for got, key in ((out.u, "u_new"), (out.v, "v_new"), (out.p, "p")):
        assert rel(got, g[key]) < TOL, (key, rel(got, g[key]))
    for grid in ("col", "mac"):
        g = golden(f"flow_gui_{grid}_{tag}")
        mac = grid == "mac"
        nx, ny = g["mask"].shape
        h = aj.StepHandler(nx, ny, float(g["dx"]), float(g["dy"]), float(g["nu"]),
                           float(g["U"]), grid_type="mac" if mac else "collocated",
                           flow_type=flow, use_les=True, les_model="smagorinsky",
                           smagorinsky_constant=float(g["cs"]), nu_hyper_ratio=float(g["hyper"]),
                           brinkman_eta=float(g["eta"]), multigrid_v_cycles=int(g["v_cycles"]),
                           sdf=None if mac else T(g["sdf"]), dt=float(g["dt"]))
        u, v, p = h._step(T(g["u"]), T(g["v"]), T(g["mask"]))
        for got, key in ((u, "u_new"), (v, "v_new"), (p, "p")):
            assert rel(got, g[key]) < TOL, (grid, key, rel(got, g[key]))
