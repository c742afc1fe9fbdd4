"""Snapshot / training-data files in the reference's format.

generate_training_data mirrors neural_operators/training_utils.py:12-81: it
runs the solver for num_steps steps and writes one .npz with float64 arrays
(num_steps, ...) for the requested fields ('u', 'v', 'p', 'mask',
'divergence') and the scalars dx, dy, dt, nx, ny.  The divergence is the
periodic central one the reference records (solver/operators.py:75-78), for
the collocated grid; on the MAC grid it is the face divergence
(solver/operators_mac.py:58-80), and u, v keep their face shapes
((nx+1, ny), (nx, ny+1)) - the reference pre-allocates (nx, ny) for them and
cannot store MAC fields.  The steps run on the GPU; each recorded field is
copied to the host once per step.
"""
from __future__ import annotations

import os
from typing import Dict, Optional

import numpy as np
import torch

from .solver import Plan, diagnostics, run_step


def generate_training_data(plan: Plan, u, v, mask, num_steps: int, save_fields: Dict[str, bool],
                           output_filename: str = "training_data.npz", p_guess=None,
                           dt: Optional[float] = None) -> str:
    cfg = plan.cfg
    mac = cfg.grid_type == "mac"
    data = {}
    shapes = {"u": tuple(u.shape), "v": tuple(v.shape), "p": (cfg.nx, cfg.ny),
              "mask": (cfg.nx, cfg.ny), "divergence": (cfg.nx, cfg.ny)}
    for k, shp in shapes.items():
        if save_fields.get(k, False):
            data[k] = np.zeros((num_steps,) + shp)
    p = p_guess if p_guess is not None else torch.zeros((cfg.nx, cfg.ny), device=u.device)
    mask_host = mask.detach().cpu().numpy().astype(np.float64)
    dts = []
    for i in range(num_steps):
        u, v, p = run_step(plan, u, v, mask, p_guess=p, dt=dt)
        dts.append(plan.stats()["dt"])
        if "u" in data:
            data["u"][i] = u.cpu().numpy()
        if "v" in data:
            data["v"][i] = v.cpu().numpy()
        if "p" in data:
            data["p"][i] = p.cpu().numpy()
        if "mask" in data:
            data["mask"][i] = mask_host
        if "divergence" in data:
            _, div, _ = diagnostics(u, v, cfg.dx, cfg.dy, grid_type=cfg.grid_type,
                                    flow_type="von_karman" if mac else "taylor_green")
            data["divergence"][i] = div.cpu().numpy()
    data["dx"] = cfg.dx
    data["dy"] = cfg.dy
    data["dt"] = dts[-1] if dts else cfg.dt
    data["nx"] = cfg.nx
    data["ny"] = cfg.ny
    np.savez(output_filename, **data)
    return os.path.abspath(output_filename)


def load_training_data(path: str) -> Dict[str, np.ndarray]:
    """The arrays of a training-data file (training_utils.py:84-110 reads
    the same keys)."""
    with np.load(path) as z:
        return {k: z[k] for k in z.files}
