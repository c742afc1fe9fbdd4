"""Trains the learned pressure warm start on snapshots the solver generates.

    python -m aerojax_gb300.train_warmstart --out aerojax_gb300/weights/<name>.npz

Snapshots (--workload naca): the NACA 0012 MAC channel (Re = 1000 on the
chord, Smagorinsky LES), angle of attack uniform in [0, 15] degrees, leading
edge shifted uniformly by up to +-64 cells (at 2048 cells); (--workload tri)
the 4096x2048 three-cylinder flow (Re = 3000, dynamic Smagorinsky,
hyperviscosity) with the triangle's centre shifted by up to +-64 cells; every
step of each run after two warm-up steps; 10 % held out
(neural_operators/training_utils.py:12-81 and :162-248 for the reference's
data flow and training loop).  Everything -
solver, features, forward and backward passes, Adam - runs in
libaerojax_gb300.so on the GPU.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import nn as NN


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="naca", choices=["naca", "tri"],
                    help="naca: NACA 0012 MAC 2048x512 family; tri: 4096x2048 three cylinders")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=512)
    ap.add_argument("--factor", type=int, default=8)
    ap.add_argument("--geoms", type=int, default=40)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    dev = torch.device("cuda:0")
    log = lambda s: print(s, flush=True)
    t0 = time.time()
    if a.workload == "naca":
        data = NN.generate_snapshots(a.nx, a.ny, n_geoms=a.geoms, steps=a.steps, factor=a.factor,
                                     seed=a.seed, device=dev, log=log)
    else:
        data = NN.generate_snapshots_tri(n_geoms=a.geoms, steps=a.steps, factor=a.factor,
                                         seed=a.seed, device=dev, log=log)
    torch.cuda.synchronize()
    t_gen = time.time() - t0
    zero_loss = float(data.target.pow(2).mean())
    log(f"{data.x3.shape[0]} snapshots in {t_gen:.1f} s; zero-prediction loss {zero_loss:.4e}")
    net = NN.WarmStartNet(device=dev, seed=a.seed)
    t0 = time.time()
    hist = NN.train(net, data, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    info = {"workload": a.workload, "nx": a.nx, "ny": a.ny, "factor": a.factor,
            "snapshots": int(data.x3.shape[0]),
            "geoms": a.geoms, "steps": a.steps, "epochs": a.epochs, "batch": a.batch, "lr": a.lr,
            "zero_prediction_loss": zero_loss, "history": hist,
            "best_heldout_loss": min(h[1] for h in hist), "generate_s": t_gen, "train_s": t_train}
    np.savez_compressed(a.out, master=net.master.cpu().numpy(), info=json.dumps(info))
    log(json.dumps(info))


if __name__ == "__main__":
    main()
