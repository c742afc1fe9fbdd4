"""The benchmark / parity workloads, built on the device.

Each builder returns a dict with the StepConfig, the mask / sdf tensors
(computed by the aj_geometry kernel) and seeded initial fields.  Sizes and
physics follow the five workloads the project is measured on:

  cylinder_512x96     collocated 512x96, lx=8, ly=1.5 (dx=dy=1/64), cylinder
                      D=16 cells at cell (96, 48), Re=150, step_pure semantics,
                      parity multigrid with 3 V-cycles, CFL 0.5
  naca_mac_2048x512   MAC 2048x512, lx=32, ly=8, NACA 0012 at 10 deg, chord 256
                      cells, leading edge at cell (400, 256), Re=1000 on the
                      chord, Smagorinsky C_s=0.17, GUI semantics, multigrid to
                      1e-6 relative residual
  tri_cyl_4096x2048   collocated 4096x2048, three cylinders D=64 cells, centre
                      spacing 160 cells, triangle centred at cell (800, 1024),
                      Re=3000 on D, dynamic Smagorinsky, hyperviscosity 0.01
Brinkman eps = eps_multiplier * dx (solver/simulation/base_solver.py:300-307),
eta from the Re presets (solver/params.py:308-413), initial u = U + 1e-3 N(0,1)
(seeded), v = 0, p = 0 (solver/simulation/initializers.py:8-30).
"""
from __future__ import annotations

import numpy as np
import torch

from .params import StepConfig, compute_eps_multiplier, get_re_parameters
from .solver import make_geometry


def _noise(shape, seed, device):
    rng = np.random.default_rng(seed)
    return torch.as_tensor(rng.standard_normal(shape).astype(np.float32), device=device)


def cylinder_512x96(device="cuda", seed=0, nx=512, ny=96, mg_mode="parity", advection="upwind",
                    cfl_dt=True):
    lx, ly = 8.0 * nx / 512, 1.5 * ny / 96
    dx, dy = lx / nx, ly / ny
    U, Re = 1.0, 150.0
    D = 16 * dx
    nu = U * D / Re
    eps = compute_eps_multiplier(Re) * dx
    cx, cy = 96 * lx / (nx - 1), (ny // 2) * ly / (ny - 1)
    mask, sdf = make_geometry("cylinder", nx, ny, lx, ly, (cx, cy, D / 2), eps, device)
    re = get_re_parameters(Re, nx)
    cfg = StepConfig(nx=nx, ny=ny, dx=dx, dy=dy, nu=nu, U_inf=U, grid_type="collocated",
                     variant="pure", advection_scheme=advection, brinkman_eta=re["brinkman_eta"],
                     v_cycles=3, mg_mode=mg_mode, has_sdf=True, cfl_dt=cfl_dt, dt=0.5 * dx,
                     cfl_target=0.5, dt_min=1e-6, dt_max=1.0, warm_start=mg_mode == "converge")
    u = 1.0 + 1e-3 * _noise((nx, ny), seed, device)
    v = torch.zeros((nx, ny), dtype=torch.float32, device=device)
    return dict(cfg=cfg, mask=mask, sdf=sdf, u=u, v=v, lx=lx, ly=ly,
                name=f"cylinder_{nx}x{ny}_collocated_re150")


def naca_mac_2048x512(device="cuda", seed=0, nx=2048, ny=512, mg_mode="converge", les=True,
                      cfl_dt=True, rtol=1e-6):
    lx, ly = 32.0 * nx / 2048, 8.0 * ny / 512
    dx, dy = lx / nx, ly / ny
    U, Re = 1.0, 1000.0
    chord = 256 * dx * nx / 2048
    nu = U * chord / Re
    eps = compute_eps_multiplier(Re) * dx
    # leading edge at (400 dx, 256 dy): placed on a grid node exactly, the
    # reference's NACA distance (obstacles/naca_airfoils.py:137-145) divides
    # 0/0 there for a symmetric section and the mask becomes NaN
    xle, yle = (400 * nx // 2048) * dx, (ny // 2) * dy
    mask, _ = make_geometry("naca4", nx, ny, lx, ly, (chord, 10.0, xle, yle, 0.0, 0.0, 0.12), eps,
                            device)
    re = get_re_parameters(Re, nx)
    cfg = StepConfig(nx=nx, ny=ny, dx=dx, dy=dy, nu=nu, U_inf=U, grid_type="mac", variant="gui",
                     use_les=les, les_model="smagorinsky", smagorinsky_constant=0.17,
                     brinkman_eta=re["brinkman_eta"], nu_hyper_ratio=re["nu_hyper_ratio"],
                     v_cycles=3, mg_mode=mg_mode, mg_rtol=rtol, max_cycles=60, cfl_dt=cfl_dt,
                     dt=0.5 * dx, cfl_target=0.5, dt_min=1e-6, dt_max=1.0,
                     warm_start=mg_mode == "converge")
    u = 1.0 + 1e-3 * _noise((nx + 1, ny), seed, device)
    v = torch.zeros((nx, ny + 1), dtype=torch.float32, device=device)
    return dict(cfg=cfg, mask=mask, sdf=None, u=u, v=v, lx=lx, ly=ly,
                name=f"naca0012_{nx}x{ny}_mac_re1000_les")


def tri_cyl_4096x2048(device="cuda", seed=0, nx=4096, ny=2048, mg_mode="converge", cfl_dt=True):
    lx, ly = 64.0 * nx / 4096, 32.0 * ny / 2048
    dx, dy = lx / nx, ly / ny
    U, Re = 1.0, 3000.0
    D = 64 * dx * nx / 4096
    nu = U * D / Re
    eps = compute_eps_multiplier(Re) * dx
    cx, cy = (800 * nx // 4096) * lx / (nx - 1), (ny // 2) * ly / (ny - 1)
    mask, sdf = make_geometry("cyl3_tri", nx, ny, lx, ly, (cx, cy, D, 160 * dx * nx / 4096), eps,
                              device)
    re = get_re_parameters(Re, nx)
    cfg = StepConfig(nx=nx, ny=ny, dx=dx, dy=dy, nu=nu, U_inf=U, grid_type="collocated",
                     variant="gui", use_les=True, les_model="dynamic_smagorinsky",
                     brinkman_eta=re["brinkman_eta"], nu_hyper_ratio=0.01, v_cycles=3,
                     mg_mode=mg_mode, max_cycles=60, has_sdf=True, cfl_dt=cfl_dt, dt=0.5 * dx,
                     cfl_target=0.5, dt_min=1e-6, dt_max=1.0, warm_start=mg_mode == "converge")
    u = 1.0 + 1e-3 * _noise((nx, ny), seed, device)
    v = torch.zeros((nx, ny), dtype=torch.float32, device=device)
    return dict(cfg=cfg, mask=mask, sdf=sdf, u=u, v=v, lx=lx, ly=ly,
                name=f"tri_cylinders_{nx}x{ny}_collocated_re3000_dynles")


def oracle_kwargs(case):
    """Keyword arguments of the oracle step matching a workload (test helper)."""
    c = case["cfg"]
    return dict(dx=c.dx, dy=c.dy, nu=c.nu, U_inf=c.U_inf, grid_type=c.grid_type,
                use_les=c.use_les, les_model=c.les_model, smagorinsky_constant=c.smagorinsky_constant,
                nu_hyper_ratio=c.nu_hyper_ratio, brinkman_eta=c.brinkman_eta, v_cycles=c.v_cycles)
