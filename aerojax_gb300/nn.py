"""Learned pressure warm start: network state, solver-generated training data,
and training — every computation runs in libaerojax_gb300.so.

The reference trains its learned pressure operators on snapshots the GUI
solver writes (neural_operators/training_utils.py:12-81) with MSE, Adam and
gradients clipped to [-1, 1], keeping the best epoch (:162-248).  Here the
network predicts a correction to the converging solve's initial guess on a
grid ``factor`` times coarser; the multigrid then finishes every solve to the
same relative residual, so the network only ever changes how many V-cycles a
step needs.  Snapshots are produced on the GPU by the solver itself and kept
in device memory.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, replace
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .params import StepConfig
from .params import compute_eps_multiplier
from .solver import Plan, _stream, get_plan, make_geometry, make_params, run_step

# the architecture table of csrc/aj_nn.cu: (Cin, Cout, relu)
LAYERS = [(16, 32, 1), (32, 32, 1), (32, 64, 1), (64, 64, 1), (64, 128, 1), (128, 128, 1),
          (128, 128, 1), (128, 128, 1), (128, 64, 1), (64, 32, 1), (32, 32, 1), (32, 16, 0)]
FEATURES = 3
# trained weights for the NACA 0012 MAC 2048x512 workload (network grid 256x64)
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                       "warmstart_naca0012_2048x512_f8.npz")
# trained weights for the 4096x2048 three-cylinder workload (network grid 512x256)
WEIGHTS_TRI = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                           "warmstart_tri_cylinders_4096x2048_f8.npz")


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights (fan-in of the live input channels), zero biases,
    the last layer scaled by 0.1 and restricted to output channel 0."""
    rng = np.random.default_rng(seed)
    parts = []
    for li, (cin, cout, _) in enumerate(LAYERS):
        fan_in = 9 * (FEATURES if li == 0 else cin)
        W = rng.standard_normal((3, 3, cin, cout)) * math.sqrt(2.0 / fan_in)
        if li == 0:
            W[:, :, FEATURES:, :] = 0.0
        if li == len(LAYERS) - 1:
            W *= 0.1
            W[:, :, :, 1:] = 0.0
        parts += [W.ravel(), np.zeros(cout)]
    return np.concatenate(parts).astype(np.float32)


class WarmStartNet:
    """FP32 master parameters, their BF16 packed copy and Adam moments."""

    def __init__(self, device="cuda", seed: int = 0, params: Optional[np.ndarray] = None):
        L = lib()
        self.n_params = int(L.aj_nn_param_count())
        self.device = torch.device(device)
        host = init_params(seed) if params is None else np.asarray(params, np.float32)
        if host.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {host.size}")
        self.master = torch.as_tensor(host, device=self.device).contiguous()
        self.packed = torch.empty(int(L.aj_nn_packed_count()), dtype=torch.int16, device=self.device)
        self.grad = torch.zeros_like(self.master)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.t = 0
        self._acts = {}
        self.pack()

    # -- parameters ----------------------------------------------------------
    def pack(self, stream=None):
        check("aj_nn_pack", lib().aj_nn_pack(self.master.data_ptr(), self.packed.data_ptr(),
                                             _stream(stream)))

    def save(self, path: str):
        np.savez_compressed(path, master=self.master.cpu().numpy(), layers=np.array(LAYERS))

    @classmethod
    def load(cls, path: str, device="cuda"):
        with np.load(path) as z:
            return cls(device=device, params=z["master"])


    # -- passes --------------------------------------------------------------
    def acts(self, n, h, w):
        key = (n, h, w)
        if key not in self._acts:
            nb = int(lib().aj_nn_act_bytes(n, h, w))
            if nb == 0:
                raise ValueError(f"network grid {h}x{w} must be a multiple of 8 in both sizes")
            self._acts[key] = torch.empty(nb, dtype=torch.uint8, device=self.device)
        return self._acts[key]

    def input_view(self, n, h, w) -> torch.Tensor:
        """The network input [n][h][w][16] inside the activation buffer."""
        buf = self.acts(n, h, w)
        ptr = lib().aj_nn_input(n, h, w, buf.data_ptr())
        off = (ptr - buf.data_ptr()) // 4
        return buf.view(torch.float32)[off:off + n * h * w * 16].view(n, h, w, 16)

    def forward(self, x16: Optional[torch.Tensor], n, h, w, stream=None) -> torch.Tensor:
        """y [n][h][w][16] (channel 0 = prediction).  x16=None uses the input
        already written into the activation buffer."""
        if x16 is not None:
            self.input_view(n, h, w).copy_(x16)
        buf = self.acts(n, h, w)
        y = torch.empty((n, h, w, 16), dtype=torch.float32, device=self.device)
        check("aj_nn_forward", lib().aj_nn_forward(n, h, w, self.packed.data_ptr(),
                                                   self.master.data_ptr(), buf.data_ptr(),
                                                   buf.numel(), y.data_ptr(), _stream(stream)))
        return y

    def backward(self, dy: torch.Tensor, n, h, w, stream=None) -> torch.Tensor:
        buf = self.acts(n, h, w)
        check("aj_nn_backward", lib().aj_nn_backward(n, h, w, dy.data_ptr(), self.packed.data_ptr(),
                                                     self.master.data_ptr(), buf.data_ptr(),
                                                     buf.numel(), self.grad.data_ptr(),
                                                     _stream(stream)))
        return self.grad

    def loss(self, y: torch.Tensor, target: torch.Tensor, n, h, w, stream=None):
        dy = torch.empty_like(y)
        loss = torch.zeros(1, dtype=torch.float64, device=self.device)
        check("aj_nn_loss", lib().aj_nn_loss(n, h, w, y.data_ptr(), target.data_ptr(),
                                             dy.data_ptr(), loss.data_ptr(), _stream(stream)))
        return loss, dy

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, clip=1.0, stream=None):
        self.t += 1
        check("aj_nn_adam", lib().aj_nn_adam(self.master.data_ptr(), self.grad.data_ptr(),
                                             self.m.data_ptr(), self.v.data_ptr(), self.t,
                                             ctypes.c_float(lr), ctypes.c_float(b1),
                                             ctypes.c_float(b2), ctypes.c_float(eps),
                                             ctypes.c_float(clip), _stream(stream)))
        self.pack(stream)

    def expand(self, x3: torch.Tensor, n, h, w, stream=None):
        """[n][h][w][3] features into the activation buffer's input."""
        dst = self.input_view(n, h, w)
        check("aj_nn_expand", lib().aj_nn_expand(n, h, w, x3.data_ptr(), dst.data_ptr(),
                                                 _stream(stream)))


# ---------------------------------------------------------------- data
@dataclass
class Snapshots:
    x3: torch.Tensor          # [N][h][w][3] normalised features
    target: torch.Tensor      # [N][h][w] normalised correction
    factor: int
    cfgs: list                # (geometry parameters) per snapshot


def naca_case(nx, ny, aoa_deg, le_shift_cells, device, factor=8, rtol=1e-6, seed=0,
              warm_start="extrapolate"):
    """The NACA 0012 MAC workload family with a given angle of attack and
    leading-edge shift (cells): the learned warm start's training geometry."""
    from . import configs
    base = configs.naca_mac_2048x512(device=device, nx=nx, ny=ny, mg_mode="converge", rtol=rtol,
                                     seed=seed)
    c = base["cfg"]
    lx, ly = base["lx"], base["ly"]
    chord = 256 * c.dx * nx / 2048
    xle = ((400 * nx // 2048) + le_shift_cells) * c.dx
    yle = (ny // 2) * c.dy
    eps = 0.05 * c.dx
    mask, _ = make_geometry("naca4", nx, ny, lx, ly, (chord, aoa_deg, xle, yle, 0.0, 0.0, 0.12),
                            eps, device)
    cfg = replace(c, nn_factor=factor, warm_start=warm_start)
    return dict(cfg=cfg, mask=mask, u=base["u"], v=base["v"])


def initial_guess(p1, p2, dt, dt1, n_hist):
    """The converging solve's initial guess under AJ_WARM_EXTRAPOLATE, in FP32:
    p1 + (dt / dt1)(p1 - p2) with two solutions in the history, p1 with one."""
    if n_hist >= 2:
        return p1 + (dt / dt1) * (p1 - p2)
    return p1.clone()


def tri_case(shift_x_cells, shift_y_cells, device, factor=8, seed=0, nx=4096, ny=2048,
             warm_start="extrapolate"):
    """The 4096x2048 three-cylinder (triangle) dynamic-LES workload with the
    triangle's centre shifted by whole cells (at 4096 cells): the second
    learned warm start's training family."""
    from . import configs
    base = configs.tri_cyl_4096x2048(device=device, nx=nx, ny=ny, seed=seed)
    c = base["cfg"]
    lx, ly = base["lx"], base["ly"]
    D = 64 * c.dx * nx / 4096
    cx = ((800 + shift_x_cells) * nx // 4096) * lx / (nx - 1)
    cy = ((ny // 2) + shift_y_cells * ny // 2048) * ly / (ny - 1)
    eps = compute_eps_multiplier(3000.0) * c.dx
    mask, sdf = make_geometry("cyl3_tri", nx, ny, lx, ly, (cx, cy, D, 160 * c.dx * nx / 4096),
                              eps, device)
    cfg = replace(c, nn_factor=factor, warm_start=warm_start)
    return dict(cfg=cfg, mask=mask, sdf=sdf, u=base["u"], v=base["v"])


def _snapshots_from(cases, n_geoms, steps, warmup, factor, device, log=None) -> Snapshots:
    """Runs the solver (extrapolated warm start) on each case and records, for
    every step after the warm-up, the network features of the step's pressure
    solve (its rhs, the mask and its initial guess) and the target correction
    (converged p minus the initial guess)."""
    x3 = tgt = None
    meta = []
    L = lib()
    k = 0
    for gidx, (case, info) in enumerate(cases):
        cfg = case["cfg"]
        nx, ny = cfg.nx, cfg.ny
        if x3 is None:
            h, w = nx // factor, ny // factor
            x3 = torch.empty((n_geoms * steps, h, w, 3), dtype=torch.float32, device=device)
            tgt = torch.empty((n_geoms * steps, h, w), dtype=torch.float32, device=device)
        plan = Plan(cfg, device)
        plan.prepare(case["mask"], case.get("sdf"))
        bufs = [(case["u"].clone(), case["v"].clone(),
                 torch.zeros((nx, ny), dtype=torch.float32, device=device)) for _ in range(2)]
        cur = 0
        hist, dts = [], []
        for s in range(warmup + steps):
            src, dst = bufs[cur], bufs[1 - cur]
            run_step(plan, src[0], src[1], case["mask"], p_guess=src[2], out=dst)
            dts.append(plan.stats()["dt"])
            if s >= max(warmup, 2) and k < x3.shape[0]:
                p_init = initial_guess(hist[-1], hist[-2], dts[-1], dts[-2], 2)
                rhs = L.aj_workspace_rhs(ctypes.byref(plan.params), plan.ws.data_ptr())
                check("aj_nn_features", L.aj_nn_features(
                    ctypes.byref(plan.params), rhs, case["mask"].data_ptr(), p_init.data_ptr(),
                    dst[2].data_ptr(), x3[k].data_ptr(), tgt[k].data_ptr(), plan.ws.data_ptr(),
                    plan.nbytes, _stream(None)))
                meta.append(info + (s,))
                k += 1
            hist = (hist + [dst[2].clone()])[-2:]
            cur = 1 - cur
        del plan
        if log:
            log(f"geometry {gidx + 1}/{n_geoms}: {info}")
    return Snapshots(x3=x3[:k], target=tgt[:k], factor=factor, cfgs=meta)


def generate_snapshots(nx=2048, ny=512, n_geoms=40, steps=500, warmup=2, factor=8, seed=0,
                       device="cuda", aoa_range=(0.0, 15.0), shift_cells=64, log=None) -> Snapshots:
    """NACA 0012 MAC snapshots: angle of attack uniform in aoa_range, leading
    edge shifted uniformly by +-shift_cells (at 2048 cells)."""
    rng = np.random.default_rng(seed)

    def cases():
        for gidx in range(n_geoms):
            aoa = float(rng.uniform(*aoa_range))
            shift = int(rng.integers(-shift_cells, shift_cells + 1)) * nx // 2048
            yield naca_case(nx, ny, aoa, shift, device, factor, seed=seed + gidx), (aoa, shift)
    return _snapshots_from(cases(), n_geoms, steps, warmup, factor, device, log)


def generate_snapshots_tri(n_geoms=8, steps=250, warmup=2, factor=8, seed=0, device="cuda",
                           shift_cells=64, nx=4096, ny=2048, log=None) -> Snapshots:
    """Three-cylinder snapshots: the triangle's centre shifted uniformly by
    +-shift_cells in x and y."""
    rng = np.random.default_rng(seed)

    def cases():
        for gidx in range(n_geoms):
            sx = int(rng.integers(-shift_cells, shift_cells + 1))
            sy = int(rng.integers(-shift_cells, shift_cells + 1))
            yield tri_case(sx, sy, device, factor, seed=seed + gidx, nx=nx, ny=ny), (sx, sy)
    return _snapshots_from(cases(), n_geoms, steps, warmup, factor, device, log)


def _last_layer_slice():
    """Offsets of the output layer's weights W[3][3][Cin][Cout] and bias in the
    flat parameter vector."""
    off = 0
    for cin, cout, _ in LAYERS[:-1]:
        off += 9 * cin * cout + cout
    cin, cout, _ = LAYERS[-1]
    return off, off + 9 * cin * cout, cin, cout


def train(net: WarmStartNet, data: Snapshots, epochs=3, batch=16, lr=1e-3, holdout=0.1, seed=0,
          log=None, normalize_target=True):
    """Adam on the MSE of the predicted correction; 10% of the snapshots held
    out; the parameters of the best held-out epoch are kept.

    normalize_target: train on target / g, g the RMS of the training targets,
    then fold g into the output layer's channel 0, so that the network
    predicts the correction in the features' units whatever its magnitude.
    If no epoch beats the zero correction on the held-out snapshots, the
    output layer is zeroed: the warm start then adds nothing (the multigrid
    judges the network's error and it has none to add).
    Returns the per-epoch (train, held-out) losses in the targets' units."""
    N, h, w, _ = data.x3.shape
    gen = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(N, generator=gen)
    n_val = max(1, int(round(N * holdout)))
    val_idx, tr_idx = perm[:n_val].to(net.device), perm[n_val:].to(net.device)
    gain = 1.0
    if normalize_target:
        gain = max(float(data.target[tr_idx].pow(2).mean().sqrt()), 1e-30)
    inv = 1.0 / gain
    zero_val = float(data.target[val_idx].pow(2).mean())
    hist = []
    best = (float("inf"), net.master.clone())

    def eval_loss(idx):
        tot, cnt = 0.0, 0
        for i in range(0, len(idx), batch):
            b = idx[i:i + batch]
            n = len(b)
            net.expand(data.x3[b].contiguous(), n, h, w)
            y = net.forward(None, n, h, w)
            loss, _ = net.loss(y, (data.target[b] * inv).contiguous(), n, h, w)
            tot += float(loss.item()) * n
            cnt += n
        return tot / max(cnt, 1) * gain * gain

    for ep in range(epochs):
        order = tr_idx[torch.randperm(len(tr_idx), generator=gen).to(net.device)]
        tl, tn = 0.0, 0
        for i in range(0, len(order) - batch + 1, batch):
            b = order[i:i + batch]
            net.expand(data.x3[b].contiguous(), batch, h, w)
            y = net.forward(None, batch, h, w)
            loss, dy = net.loss(y, (data.target[b] * inv).contiguous(), batch, h, w)
            net.backward(dy, batch, h, w)
            net.adam(lr=lr)
            tl += float(loss.item())
            tn += 1
        vl = eval_loss(val_idx)
        hist.append((tl / max(tn, 1) * gain * gain, vl))
        if vl < best[0]:
            best = (vl, net.master.clone())
        if log:
            log(f"epoch {ep + 1}/{epochs}: train {hist[-1][0]:.4e}  held-out {vl:.4e}  "
                f"(zero correction {zero_val:.4e})")
    master = best[1].cpu().numpy().copy()
    w0, b0, cin, cout = _last_layer_slice()
    W = master[w0:b0].reshape(3, 3, cin, cout)
    if best[0] >= zero_val:
        W[..., 0] = 0.0
        master[b0] = 0.0
        if log:
            log("no epoch beats the zero correction on the held-out snapshots: output layer zeroed")
    else:
        W[..., 0] *= gain
        master[b0] *= gain
    master[w0:b0] = W.ravel()
    net.master.copy_(torch.as_tensor(master, device=net.device))
    net.pack()
    return hist


def warm_start_guess(plan: Plan, net: WarmStartNet, rhs, mask, p_prev, out=None, stream=None):
    """The learned warm start on its own (aj_nn_warmstart): p0 = p_prev + the
    network's correction from (rhs, mask, p_prev) - the guess to hand to
    poisson_multigrid_converge(..., p0=p0).  plan: a converging-mode plan
    with nn_factor set (its workspace holds the network's activations)."""
    cfg = plan.cfg
    p0 = out if out is not None else torch.empty((cfg.nx, cfg.ny), dtype=torch.float32,
                                                 device=rhs.device)
    check("aj_nn_warmstart", lib().aj_nn_warmstart(
        ctypes.byref(plan.params), rhs.data_ptr(), mask.data_ptr(), p_prev.data_ptr(),
        net.packed.data_ptr(), net.master.data_ptr(), p0.data_ptr(), plan.ws.data_ptr(),
        plan.nbytes, _stream(stream)))
    return p0


def run_step_nn(plan: Plan, net: WarmStartNet, u, v, mask, p_prev, out=None, stream=None):
    """One step whose pressure solve starts from the plan's initial guess
    (p_prev, or the extrapolation of the workspace's history) plus the
    network's correction (aj_step_nn); returns (u, v, p)."""
    cfg = plan.cfg
    if out is None:
        out = (torch.empty_like(u), torch.empty_like(v),
               torch.empty((cfg.nx, cfg.ny), dtype=torch.float32, device=u.device))
    uo, vo, po = out
    check("aj_step_nn", lib().aj_step_nn(ctypes.byref(plan.params), u.data_ptr(), v.data_ptr(),
                                         mask.data_ptr(), p_prev.data_ptr(), net.packed.data_ptr(),
                                         net.master.data_ptr(), uo.data_ptr(), vo.data_ptr(),
                                         po.data_ptr(), plan.ws.data_ptr(), plan.nbytes,
                                         plan.stats_buf.data_ptr(), _stream(stream)))
    return uo, vo, po
