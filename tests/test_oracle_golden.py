"""The oracle against the golden fixtures made by running the reference's own
source files (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import golden
from oracle import ref_np as R


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


TOL = 1e-12   # same algorithm in float64: only summation order may differ


@pytest.mark.parametrize("name", ["mg_64x32", "mg_128x48"])
def test_multigrid(name):
    g = golden(name)
    p = R.poisson_multigrid(g["rhs"], g["mask"], float(g["dx"]), float(g["dy"]),
                            v_cycles=int(g["v_cycles"]))
    pm = R.poisson_multigrid_mac(g["rhs"], g["mask"], float(g["dx"]), float(g["dy"]),
                                 v_cycles=int(g["v_cycles"]))
    assert rel(p, g["p"]) < TOL
    assert rel(pm, g["p_mac"]) < TOL


@pytest.mark.parametrize("name", ["rk3", "rk2", "rk3_hyper", "rk3_field"])
def test_predictor_collocated(name):
    g = golden("pred_" + name)
    nu = g["nu"] if g["nu"].ndim else float(g["nu"])
    nsg = None if g["nu_sgs"].shape == (1, 1) else g["nu_sgs"]
    us, vs = R.rk_step_unified(g["u"], g["v"], float(g["dt"]), nu, float(g["dx"]), float(g["dy"]),
                               g["mask"], sdf=g["sdf"], U_inf=float(g["U"]), nu_sgs=nsg,
                               nu_hyper_ratio=float(g["hyper"]), fast_mode=bool(g["fast"]),
                               brinkman_eta=float(g["eta"]))
    assert rel(us, g["u_star"]) < TOL and rel(vs, g["v_star"]) < TOL


@pytest.mark.parametrize("name", ["mac_rk3", "mac_rk2_les_hyper"])
def test_predictor_mac(name):
    g = golden("pred_" + name)
    nsg = None if g["nu_sgs"].shape == (1, 1) else g["nu_sgs"]
    us, vs = R.rk_step_unified_mac(g["u"], g["v"], float(g["dt"]), float(g["nu"]), float(g["dx"]),
                                   float(g["dy"]), g["mask"], U_inf=float(g["U"]), nu_sgs=nsg,
                                   nu_hyper_ratio=float(g["hyper"]), fast_mode=bool(g["fast"]),
                                   brinkman_eta=float(g["eta"]))
    assert rel(us, g["u_star"]) < TOL and rel(vs, g["v_star"]) < TOL


def test_les():
    g = golden("les")
    c = R.constant_smagorinsky(g["u"], g["v"], float(g["dx"]), float(g["dy"]), float(g["delta"]), 0.17)
    d, cd = R.dynamic_smagorinsky(g["u"], g["v"], float(g["dx"]), float(g["dy"]), float(g["delta"]))
    assert rel(c, g["nu_const"]) < TOL
    assert rel(d, g["nu_dyn"]) < TOL and rel(cd, g["cd"]) < TOL


def test_step_pure():
    g = golden("step_pure")
    un, vn, p = R.step_pure(g["u"], g["v"], float(g["dt"]), g["mask"], g["sdf"], float(g["dx"]),
                            float(g["dy"]), float(g["nu"]), float(g["U"]), v_cycles=3,
                            brinkman_eta=float(g["eta"]))
    assert rel(un, g["u_new"]) < TOL and rel(vn, g["v_new"]) < TOL and rel(p, g["p"]) < TOL


@pytest.mark.parametrize("name", ["gui_col_les", "gui_col_dyn", "gui_col_plain", "gui_mac_les",
                                  "gui_mac_plain"])
def test_step_gui(name):
    g = golden("step_" + name)
    mac = "mac" in name
    un, vn, p = R.step_gui(g["u"], g["v"], g["mask"], float(g["dt"]),
                           sdf=None if mac else g["sdf"], dx=float(g["dx"]), dy=float(g["dy"]),
                           nu=float(g["nu"]), U_inf=float(g["U"]),
                           grid_type="mac" if mac else "collocated", use_les=bool(g["use_les"]),
                           les_model="dynamic_smagorinsky" if int(g["dynamic"]) else "smagorinsky",
                           smagorinsky_constant=float(g["cs"]), nu_hyper_ratio=float(g["hyper"]),
                           brinkman_eta=float(g["eta"]), v_cycles=int(g["v_cycles"]))
    assert rel(un, g["u_new"]) < TOL and rel(vn, g["v_new"]) < TOL and rel(p, g["p"]) < TOL


def test_cfl():
    g = golden("cfl")
    a = R.compute_cfl_timestep(g["u"], g["v"], float(g["dx"]), float(g["dy"]), float(g["nu"]),
                               0.5, 1e-5, 0.05)
    b = R.compute_cfl_timestep(g["um"], g["vm"], float(g["dx"]), float(g["dy"]), float(g["nu"]),
                               0.5, 1e-5, 0.05)
    assert a == pytest.approx(float(g["dt"]), rel=1e-14)
    assert b == pytest.approx(float(g["dt_mac"]), rel=1e-14)


def test_geometry():
    g = golden("geometry")
    s = R.sdf_naca4(g["X"], g["Y"], 1.5, 10.0, 1.5, 1.5, 0.0, 0.0, 0.12)
    assert np.array_equal(np.isnan(s), np.isnan(g["sdf_naca0012"]))
    assert np.nanmax(np.abs(s - g["sdf_naca0012"])) < 1e-13
    s2 = R.sdf_naca4(g["X"], g["Y"], 1.5, 5.0, 1.5, 1.5, 0.02, 0.4, 0.12)
    assert np.nanmax(np.abs(s2 - g["sdf_naca2412"])) < 1e-13
    s3 = R.sdf_three_cylinders_inline(g["X"], g["Y"], 2.0, 1.5, 0.5, 0.8)
    assert np.max(np.abs(s3 - g["sdf_three"])) < 1e-13


def test_scalar_advection_matches_reference():
    """The dye step (operators.py:111-150, operators_mac.py:161-215), all four
    grid/flow variants, bit for bit in float64."""
    z = golden("scalar")
    a = (float(z["dt"]), float(z["dx"]), float(z["dy"]), float(z["kappa"]))
    for mac, u, v in ((False, z["u"], z["v"]), (True, z["um"], z["vm"])):
        for per in (False, True):
            c = R.scalar_advection_diffusion(z["c"], u, v, a[0], a[1], a[2], a[3], mac=mac,
                                             periodic=per)
            tag = ("mac_" if mac else "col_") + ("per" if per else "np")
            assert np.array_equal(c, z[tag]), tag


def test_diagnostics_match_reference():
    """Vorticity and divergence of step_for_visualization
    (visualization_step.py:224-256), all four grid/flow variants."""
    z = golden("diagnostics")
    dx, dy = float(z["dx"]), float(z["dy"])
    for mac, u, v in ((False, z["u"], z["v"]), (True, z["um"], z["vm"])):
        for per in (False, True):
            vort, div, _ = R.diagnostics(u, v, dx, dy, mac=mac, periodic=per)
            tag = ("mac_" if mac else "") + ("per" if per else "np")
            assert np.array_equal(vort, z["vort_" + tag]), tag
            assert np.allclose(div, z["div_" + tag], rtol=0, atol=1e-12), tag


@pytest.mark.parametrize("tag", ["ldc", "tg"])
def test_other_flow_types(tag):
    """Lid-driven cavity and Taylor-Green: the reference's multigrid (mean
    subtraction, wrapped residual), step_pure and both GUI steps with that
    flow type, run from its own source (fixtures flow_*)."""
    g = golden(f"flow_mg_{tag}")
    flow = str(g["flow"])
    p = R.poisson_multigrid(g["rhs"], g["mask"], float(g["dx"]), float(g["dy"]),
                            v_cycles=int(g["v_cycles"]), flow_type=flow)
    pm = R.poisson_multigrid_mac(g["rhs"], g["mask"], float(g["dx"]), float(g["dy"]),
                                 v_cycles=int(g["v_cycles"]), flow_type=flow)
    assert rel(p, g["p"]) < TOL and rel(pm, g["p_mac"]) < TOL
    g = golden(f"flow_step_pure_{tag}")
    un, vn, pn = R.step_pure(g["u"], g["v"], float(g["dt"]), g["mask"], g["sdf"], float(g["dx"]),
                             float(g["dy"]), float(g["nu"]), float(g["U"]),
                             v_cycles=int(g["v_cycles"]), brinkman_eta=float(g["eta"]),
                             flow_type=flow)
    assert rel(un, g["u_new"]) < TOL and rel(vn, g["v_new"]) < TOL and rel(pn, g["p"]) < TOL
    for grid in ("col", "mac"):
        g = golden(f"flow_gui_{grid}_{tag}")
        mac = grid == "mac"
        un, vn, pn = R.step_gui(g["u"], g["v"], g["mask"], float(g["dt"]),
                                sdf=None if mac else g["sdf"], dx=float(g["dx"]),
                                dy=float(g["dy"]), nu=float(g["nu"]), U_inf=float(g["U"]),
                                grid_type="mac" if mac else "collocated", use_les=True,
                                les_model="smagorinsky", smagorinsky_constant=float(g["cs"]),
                                nu_hyper_ratio=float(g["hyper"]), brinkman_eta=float(g["eta"]),
                                v_cycles=int(g["v_cycles"]), flow_type=flow)
        for a, key in ((un, "u_new"), (vn, "v_new"), (pn, "p")):
            assert rel(a, g[key]) < TOL, (grid, key, rel(a, g[key]))
