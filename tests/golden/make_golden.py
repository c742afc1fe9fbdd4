"""Generate the golden fixtures by running the reference's own source files.

The AeroJAX reference is pure Python/JAX; jax is not installed in this
container, so its files are executed under ``jax_numpy_shim`` (a NumPy
stand-in for the jax API, float64).  Nothing here is imported by the product
or by the GPU tests; the fixtures it writes (``tests/golden/*.npz``) are what
travels.

Usage:  python tests/golden/make_golden.py REFERENCE_ROOT
(or set $AEROJAX_REF to the AeroJAX checkout and omit the argument;
$AEROJAX_GOLDEN_ONLY=prefix writes only the fixtures whose names start with it).
"""
from __future__ import annotations

import importlib
import os
import sys
import types
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import jax_numpy_shim  # noqa: E402


def load_reference(root):
    jax_numpy_shim.install()
    sys.path.insert(0, root)

    def pkg(name, rel):
        m = types.ModuleType(name)
        m.__path__ = [os.path.join(root, rel)]
        sys.modules[name] = m
        return m

    # packages whose __init__ pulls in the GUI are replaced by bare stubs
    solver = pkg("solver", "solver")
    pf = pkg("solver.pure_functions", "solver/pure_functions")
    pkg("solver.simulation", "solver/simulation")
    ps = pkg("pressure_solvers", "pressure_solvers")
    pkg("advection_schemes", "advection_schemes")
    pkg("timestepping", "timestepping")
    pkg("obstacles", "obstacles")
    sys.modules["pressure_solvers.cg"] = None      # optional solvers: ImportError
    sys.modules["pressure_solvers.FFT"] = None
    mg = importlib.import_module("pressure_solvers.multigrid_solver")
    ps.poisson_multigrid, ps.poisson_jacobi = mg.poisson_multigrid, mg.poisson_jacobi
    mods = SimpleNamespace(mg=mg)
    mods.mgm = importlib.import_module("pressure_solvers.multigrid_solver_mac")
    mods.ops = importlib.import_module("solver.operators")
    mods.opsm = importlib.import_module("solver.operators_mac")
    mods.les = importlib.import_module("solver.les_models")
    mods.params = importlib.import_module("solver.params")
    mods.rk = importlib.import_module("advection_schemes.rk3_simple_new")
    mods.rkm = importlib.import_module("advection_schemes.rk3_mac")
    mods.corner = importlib.import_module("solver.pure_functions.corner_smoothing")
    mods.dtc = importlib.import_module("solver.pure_functions.dt_controller")
    pf.apply_corner_smooth_pressure_gradient = mods.corner.apply_corner_smooth_pressure_gradient
    pf.apply_corner_smooth_inlet = mods.corner.apply_corner_smooth_inlet
    pf.update_dt_pure = mods.dtc.update_dt_pure
    mods.step = importlib.import_module("solver.pure_functions.step")
    pf.step_pure = mods.step.step_pure
    mods.bcs = importlib.import_module("solver.boundary_conditions")
    mods.sh = importlib.import_module("solver.simulation.step_handlers")
    mods.cfl = importlib.import_module("timestepping.cfl_adaptive_dt")
    mods.naca = importlib.import_module("obstacles.naca_airfoils")
    mods.cyl = importlib.import_module("obstacles.cylinder_array")
    return mods


def flow_case(nx, ny, lx, ly, seed, noise=1e-2, cyl=(0.25, 0.5, 0.125)):
    """Seeded inlet-like velocity field, cylinder mask/sdf; float64."""
    rng = np.random.default_rng(seed)
    dx, dy = lx / nx, ly / ny
    x = np.linspace(0, lx, nx)
    y = np.linspace(0, ly, ny)
    X, Y = np.meshgrid(x, y, indexing="ij")
    cx, cy, r = cyl[0] * lx, cyl[1] * ly, cyl[2] * ly
    sdf = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2) - r
    eps = 0.05 * dx
    mask = 1.0 - 1.0 / (1.0 + np.exp(np.clip(sdf / eps, -700, 700)))
    u = 1.0 + noise * rng.standard_normal((nx, ny))
    v = noise * rng.standard_normal((nx, ny))
    # a few smooth eddies so that advection, LES and the projection all act
    u += 0.2 * np.sin(2 * np.pi * X / lx) * np.cos(2 * np.pi * Y / ly)
    v += 0.2 * np.cos(2 * np.pi * X / lx) * np.sin(2 * np.pi * Y / ly)
    return dict(u=u, v=v, mask=mask, sdf=sdf, dx=dx, dy=dy, X=X, Y=Y)


def mac_fields(c, seed):
    rng = np.random.default_rng(seed)
    nx, ny = c["u"].shape
    um = np.empty((nx + 1, ny))
    um[:-1] = c["u"]
    um[-1] = c["u"][-1]
    vm = np.empty((nx, ny + 1))
    vm[:, :-1] = c["v"]
    vm[:, -1] = 0.0
    um += 1e-3 * rng.standard_normal(um.shape)
    return um, vm


def fake_solver(c, *, nu, U, grid_type, use_les, les_model, cs, hyper, eta, v_cycles, dt,
                fast_mode=False):
    nx, ny = c["u"].shape
    s = SimpleNamespace()
    s.grid = SimpleNamespace(dx=c["dx"], dy=c["dy"], nx=nx, ny=ny)
    s.flow = SimpleNamespace(nu=nu, U_inf=U)
    s.sim_params = SimpleNamespace(use_les=use_les, les_model=les_model, smagorinsky_constant=cs,
                                   fast_mode=fast_mode, brinkman_eta=eta, flow_type="von_karman",
                                   pressure_solver="multigrid", multigrid_v_cycles=v_cycles,
                                   grid_type=grid_type, pressure_max_iter=50,
                                   pressure_tolerance=1e-10)
    s.sdf = J(c["sdf"])
    s.nu_hyper_ratio = hyper
    s.slip_walls = True
    s.nn_pressure_model = None
    s.dt = dt
    s.iteration = 5
    s.startup_ramp_steps = 0
    return s


def A(x):
    return np.asarray(x, dtype=np.float64)


def J(x):
    return np.asarray(x, dtype=np.float64).view(jax_numpy_shim.JArr)


def main(root):
    R = load_reference(root)
    out = {}

    # --- multigrid, collocated and MAC (parity mode) -------------------------
    for (nx, ny, seed, vc) in [(64, 32, 1, 3), (128, 48, 2, 5)]:
        c = flow_case(nx, ny, 4.0, 2.0 * ny / 32, seed)
        rng = np.random.default_rng(seed + 100)
        rhs = rng.standard_normal((nx, ny)) * 10.0
        p = R.mg.poisson_multigrid(rhs, c["mask"], c["dx"], c["dy"], v_cycles=vc)
        pm = R.mgm.poisson_multigrid_mac(rhs, c["mask"], c["dx"], c["dy"], v_cycles=vc)
        out[f"mg_{nx}x{ny}"] = dict(rhs=rhs, mask=c["mask"], dx=c["dx"], dy=c["dy"], v_cycles=vc,
                                    p=A(p), p_mac=A(pm))

    # --- predictors ------------------------------------------------------------
    c = flow_case(64, 32, 4.0, 2.0, 3)
    dt, nu, U = 4e-3, 0.01, 1.0
    nu_field = nu + 1e-3 * np.abs(np.random.default_rng(7).standard_normal((64, 32)))
    cases = {
        "rk3": dict(nu=nu, nu_sgs=None, hyper=0.0, fast=False),
        "rk2": dict(nu=nu, nu_sgs=None, hyper=0.0, fast=True),
        "rk3_hyper": dict(nu=nu, nu_sgs=None, hyper=0.01, fast=False),
        "rk3_field": dict(nu=nu_field, nu_sgs=nu_field - nu, hyper=0.01, fast=False),
    }
    for name, k in cases.items():
        us, vs = R.rk.rk_step_unified(c["u"], c["v"], dt, k["nu"], c["dx"], c["dy"], c["mask"],
                                      sdf=c["sdf"], U_inf=U, nu_sgs=k["nu_sgs"],
                                      nu_hyper_ratio=k["hyper"], slip_walls=True,
                                      fast_mode=k["fast"], brinkman_eta=1e-3,
                                      flow_type="von_karman")
        out[f"pred_{name}"] = dict(u=c["u"], v=c["v"], mask=c["mask"], sdf=c["sdf"], dx=c["dx"],
                                   dy=c["dy"], dt=dt, nu=k["nu"],
                                   nu_sgs=(np.zeros((1, 1)) if k["nu_sgs"] is None else k["nu_sgs"]),
                                   hyper=k["hyper"], fast=int(k["fast"]), eta=1e-3, U=U,
                                   u_star=A(us), v_star=A(vs))
    um, vm = mac_fields(c, 4)
    for name, (nsg, hyper, fast) in {"mac_rk3": (None, 0.0, False),
                                     "mac_rk2_les_hyper": ("les", 0.01, True)}.items():
        nu_sgs = None
        if nsg:
            uc, vc_ = R.opsm.interpolate_to_cell_center(um, vm)
            nu_sgs = A(R.les.constant_smagorinsky(uc, vc_, c["dx"], c["dy"],
                                                  (c["dx"] * c["dy"]) ** 0.5, 0.17))
        us, vs = R.rkm.rk_step_unified_mac(um, vm, dt, nu, c["dx"], c["dy"], c["mask"], U_inf=U,
                                           nu_sgs=nu_sgs, nu_hyper_ratio=hyper, slip_walls=True,
                                           fast_mode=fast, brinkman_eta=1e-3,
                                           flow_type="von_karman")
        out[f"pred_{name}"] = dict(u=um, v=vm, mask=c["mask"], dx=c["dx"], dy=c["dy"], dt=dt,
                                   nu=nu, nu_sgs=(np.zeros((1, 1)) if nu_sgs is None else nu_sgs),
                                   hyper=hyper, fast=int(fast), eta=1e-3, U=U,
                                   u_star=A(us), v_star=A(vs))

    # --- LES -------------------------------------------------------------------
    delta = (c["dx"] * c["dy"]) ** 0.5
    nus_c = R.les.constant_smagorinsky(c["u"], c["v"], c["dx"], c["dy"], delta, 0.17)
    nus_d, cd = R.les.dynamic_smagorinsky(c["u"], c["v"], c["dx"], c["dy"], delta)
    out["les"] = dict(u=c["u"], v=c["v"], dx=c["dx"], dy=c["dy"], delta=delta, cs=0.17,
                      nu_const=A(nus_c), nu_dyn=A(nus_d), cd=A(cd))

    # --- full steps --------------------------------------------------------------
    st = R.params.SimState(u=c["u"], v=c["v"], p=np.zeros((64, 32)), u_prev=c["u"], v_prev=c["v"],
                           c=np.zeros((64, 32)), dt=dt, iteration=0)
    res = R.step.step_pure(st, c["mask"], c["sdf"], c["dx"], c["dy"], nu, U, v_cycles=3,
                           brinkman_eta=1e-3)
    out["step_pure"] = dict(u=c["u"], v=c["v"], mask=c["mask"], sdf=c["sdf"], dx=c["dx"],
                            dy=c["dy"], dt=dt, nu=nu, U=U, eta=1e-3, v_cycles=3,
                            u_new=A(res.u), v_new=A(res.v), p=A(res.p))
    for name, kw in {
        "gui_col_les": dict(grid_type="collocated", use_les=True, les_model="smagorinsky",
                            cs=0.17, hyper=0.01),
        "gui_col_dyn": dict(grid_type="collocated", use_les=True,
                            les_model="dynamic_smagorinsky", cs=0.17, hyper=0.0),
        "gui_col_plain": dict(grid_type="collocated", use_les=False, les_model="smagorinsky",
                              cs=0.17, hyper=0.0),
    }.items():
        s = fake_solver(c, nu=nu, U=U, eta=1e-3, v_cycles=3, dt=dt, **kw)
        un, vn, p = R.sh._step_collocated(s, J(c["u"]), J(c["v"]), J(c["mask"]), dt)
        out[f"step_{name}"] = dict(u=c["u"], v=c["v"], mask=c["mask"], sdf=c["sdf"],
                                   dx=c["dx"], dy=c["dy"], dt=dt, nu=nu, U=U, eta=1e-3,
                                   v_cycles=3, use_les=int(kw["use_les"]),
                                   dynamic=int(kw["les_model"] == "dynamic_smagorinsky"),
                                   cs=kw["cs"], hyper=kw["hyper"],
                                   u_new=A(un), v_new=A(vn), p=A(p))
    for name, kw in {
        "gui_mac_les": dict(use_les=True, les_model="smagorinsky", cs=0.17, hyper=0.0),
        "gui_mac_plain": dict(use_les=False, les_model="smagorinsky", cs=0.17, hyper=0.01),
    }.items():
        s = fake_solver(c, nu=nu, U=U, eta=1e-3, v_cycles=3, dt=dt, grid_type="mac", **kw)
        un, vn, p = R.sh._step_mac(s, J(um), J(vm), J(c["mask"]), dt)
        out[f"step_{name}"] = dict(u=um, v=vm, mask=c["mask"], dx=c["dx"], dy=c["dy"], dt=dt,
                                   nu=nu, U=U, eta=1e-3, v_cycles=3,
                                   use_les=int(kw["use_les"]), dynamic=0, cs=kw["cs"],
                                   hyper=kw["hyper"], u_new=A(un), v_new=A(vn), p=A(p))

    # --- post-step diagnostics (visualization_step.py:224-256) ------------------
    out["diagnostics"] = dict(
        u=c["u"], v=c["v"], um=um, vm=vm, dx=c["dx"], dy=c["dy"],
        vort_np=A(R.ops.vorticity_nonperiodic(c["u"], c["v"], c["dx"], c["dy"])),
        div_np=A(R.ops.divergence_nonperiodic(c["u"], c["v"], c["dx"], c["dy"])),
        vort_per=A(R.ops.vorticity(c["u"], c["v"], c["dx"], c["dy"])),
        div_per=A(R.ops.divergence(c["u"], c["v"], c["dx"], c["dy"])),
        vort_mac_np=A(R.opsm.vorticity_nonperiodic_staggered(um, vm, c["dx"], c["dy"])),
        div_mac_np=A(R.opsm.divergence_nonperiodic_staggered(um, vm, c["dx"], c["dy"])),
        vort_mac_per=A(R.opsm.vorticity_staggered(um, vm, c["dx"], c["dy"])),
        div_mac_per=A(R.opsm.divergence_staggered(um, vm, c["dx"], c["dy"])))

    # --- passive scalar (dye) advection-diffusion (operators.py:111-150,
    # operators_mac.py:161-215) --------------------------------------------------
    rng = np.random.default_rng(7)
    nxs, nys = c["u"].shape
    X, Y = np.meshgrid(np.linspace(0, 1, nxs), np.linspace(0, 1, nys), indexing="ij")
    dye = np.clip(np.exp(-((X - 0.3) ** 2 + (Y - 0.5) ** 2) / 0.02)
                  + 0.05 * rng.standard_normal(X.shape), 0.0, 1.0)
    dts, kap = 0.004, 0.002
    out["scalar"] = dict(
        c=dye, u=c["u"], v=c["v"], um=um, vm=vm, dx=c["dx"], dy=c["dy"], dt=dts, kappa=kap,
        col_per=A(R.ops.scalar_advection_diffusion_periodic(dye, c["u"], c["v"], dts, c["dx"],
                                                            c["dy"], kap)),
        col_np=A(R.ops.scalar_advection_diffusion_nonperiodic(dye, c["u"], c["v"], dts, c["dx"],
                                                              c["dy"], kap)),
        mac_per=A(R.opsm.scalar_advection_diffusion_periodic_staggered(dye, um, vm, dts, c["dx"],
                                                                       c["dy"], kap)),
        mac_np=A(R.opsm.scalar_advection_diffusion_nonperiodic_staggered(dye, um, vm, dts,
                                                                         c["dx"], c["dy"], kap)))

    # --- time step and geometry ---------------------------------------------------
    dtc = R.cfl.compute_cfl_timestep(c["u"], c["v"], c["dx"], c["dy"], nu, cfl_target=0.5,
                                     dt_min=1e-5, dt_max=0.05)
    dtm = R.cfl.compute_cfl_timestep(um, vm, c["dx"], c["dy"], nu, cfl_target=0.5,
                                     dt_min=1e-5, dt_max=0.05)
    out["cfl"] = dict(u=c["u"], v=c["v"], um=um, vm=vm, dx=c["dx"], dy=c["dy"], nu=nu,
                      dt=float(dtc), dt_mac=float(dtm))
    nx, ny, lx, ly = 96, 48, 6.0, 3.0
    X, Y = np.meshgrid(np.linspace(0, lx, nx), np.linspace(0, ly, ny), indexing="ij")
    m, p_, t = R.naca.parse_naca_4digit("0012")
    sdf_n = R.naca.naca_surface_distance(X, Y, 1.5, 10.0, 1.5, 1.5, m, p_, t)
    m2, p2, t2 = R.naca.parse_naca_4digit("2412")
    sdf_n2 = R.naca.naca_surface_distance(X, Y, 1.5, 5.0, 1.5, 1.5, m2, p2, t2)
    sdf_3 = R.cyl.sdf_three_cylinders(X, Y, 2.0, 1.5, 0.5, 0.8)
    out["geometry"] = dict(X=X, Y=Y, sdf_naca0012=A(sdf_n), sdf_naca2412=A(sdf_n2),
                           sdf_three=A(sdf_3))

    # --- the other flow types: lid-driven cavity and Taylor-Green -----------------
    # (multigrid_solver.py:75-80 and :173-183, step.py:259-264 and :378-390,
    # step_handlers.py:129-183 / :240-274 with sim_params.flow_type)
    for flow, tag in (("lid_driven_cavity", "ldc"), ("taylor_green", "tg")):
        cm = flow_case(64, 32, 4.0, 2.0, 1)
        rhs = np.random.default_rng(11).standard_normal((64, 32)) * 10.0
        p = R.mg.poisson_multigrid(rhs, cm["mask"], cm["dx"], cm["dy"], v_cycles=3, flow_type=flow)
        pm = R.mgm.poisson_multigrid_mac(rhs, cm["mask"], cm["dx"], cm["dy"], v_cycles=3,
                                         flow_type=flow)
        out[f"flow_mg_{tag}"] = dict(rhs=rhs, mask=cm["mask"], dx=cm["dx"], dy=cm["dy"],
                                     v_cycles=3, flow=flow, p=A(p), p_mac=A(pm))
        st = R.params.SimState(u=c["u"], v=c["v"], p=np.zeros((64, 32)), u_prev=c["u"],
                               v_prev=c["v"], c=np.zeros((64, 32)), dt=dt, iteration=0)
        res = R.step.step_pure(st, c["mask"], c["sdf"], c["dx"], c["dy"], nu, U, v_cycles=3,
                               brinkman_eta=1e-3, flow_type=flow)
        out[f"flow_step_pure_{tag}"] = dict(u=c["u"], v=c["v"], mask=c["mask"], sdf=c["sdf"],
                                            dx=c["dx"], dy=c["dy"], dt=dt, nu=nu, U=U, eta=1e-3,
                                            v_cycles=3, flow=flow, u_new=A(res.u),
                                            v_new=A(res.v), p=A(res.p))
        s = fake_solver(c, nu=nu, U=U, eta=1e-3, v_cycles=3, dt=dt, grid_type="collocated",
                        use_les=True, les_model="smagorinsky", cs=0.17, hyper=0.01)
        s.sim_params.flow_type = flow
        un, vn, p = R.sh._step_collocated(s, J(c["u"]), J(c["v"]), J(c["mask"]), dt)
        out[f"flow_gui_col_{tag}"] = dict(u=c["u"], v=c["v"], mask=c["mask"], sdf=c["sdf"],
                                          dx=c["dx"], dy=c["dy"], dt=dt, nu=nu, U=U, eta=1e-3,
                                          v_cycles=3, use_les=1, dynamic=0, cs=0.17, hyper=0.01,
                                          flow=flow, u_new=A(un), v_new=A(vn), p=A(p))
        s = fake_solver(c, nu=nu, U=U, eta=1e-3, v_cycles=3, dt=dt, grid_type="mac",
                        use_les=True, les_model="smagorinsky", cs=0.17, hyper=0.0)
        s.sim_params.flow_type = flow
        un, vn, p = R.sh._step_mac(s, J(um), J(vm), J(c["mask"]), dt)
        out[f"flow_gui_mac_{tag}"] = dict(u=um, v=vm, mask=c["mask"], dx=c["dx"], dy=c["dy"],
                                          dt=dt, nu=nu, U=U, eta=1e-3, v_cycles=3, use_les=1,
                                          dynamic=0, cs=0.17, hyper=0.0, flow=flow, u_new=A(un),
                                          v_new=A(vn), p=A(p))

    only = os.environ.get("AEROJAX_GOLDEN_ONLY", "")
    n = 0
    for name, d in out.items():
        if only and not name.startswith(only):
            continue
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        n += 1
    print(f"wrote {n} fixtures to {HERE}")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AEROJAX_REF")
    if not root:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set AEROJAX_REF)")
    main(root)
