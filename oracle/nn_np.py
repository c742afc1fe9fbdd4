"""CPU oracle of the learned pressure warm start — TEST INFRASTRUCTURE ONLY.

NumPy float64 forward and backward of the encoder-decoder that predicts a
pressure correction (imported only by tests/ and bench.py's CPU legs).  The
reference's learned operators (neural_operators/nn_pressure_operator_*.py)
replace the pressure solve; this network instead warm-starts the multigrid,
which always finishes the solve.  The data contract follows the reference:
per-sample channel normalisation of the inputs
(neural_operators/nn_pressure_operator_advanced.py:56-59), 3x3 'SAME'
cross-correlation convolutions with zero padding, ReLU, MSE loss and Adam
with gradients clipped to [-1, 1] (neural_operators/training_utils.py:170-188).

Architecture (shared with aerojax_gb300/csrc/aj_nn.cu; activations NHWC):
  e0a 16->32, e0b 32->32 (s0) | pool | e1a 32->64, e1b 64->64 (s1) | pool |
  e2a 64->128, e2b 128->128 (s2) | pool | e3a 128->128, e3b 128->128 |
  up + s2 | d2 128->64 | up + s1 | d1 64->32 | up + s0 | d0a 32->32 |
  d0b 32->16 (linear; channel 0 is the output)
Input channels 0..2 carry the features, 3..15 are zero; output channels 1..15
carry zero weights.  Every conv has a bias; all but d0b apply ReLU.
"""
from __future__ import annotations

import numpy as np

# (name, Cin, Cout, relu)
LAYERS = [
    ("e0a", 16, 32, True), ("e0b", 32, 32, True),
    ("e1a", 32, 64, True), ("e1b", 64, 64, True),
    ("e2a", 64, 128, True), ("e2b", 128, 128, True),
    ("e3a", 128, 128, True), ("e3b", 128, 128, True),
    ("d2", 128, 64, True), ("d1", 64, 32, True),
    ("d0a", 32, 32, True), ("d0b", 32, 16, False),
]
IN_CH, OUT_CH, FEATURES = 16, 16, 3


def param_shapes():
    return [(name, (3, 3, cin, cout), (cout,)) for name, cin, cout, _ in LAYERS]


def num_params():
    return sum(9 * cin * cout + cout for _, cin, cout, _ in LAYERS)


def unflatten(flat):
    """Flat FP32 parameter vector -> {name: (W[3][3][Cin][Cout], b[Cout])};
    order: for each layer, W (tap-major, then Cin, then Cout), then b."""
    out, o = {}, 0
    for name, cin, cout, _ in LAYERS:
        n = 9 * cin * cout
        W = flat[o:o + n].reshape(3, 3, cin, cout)
        o += n
        b = flat[o:o + cout]
        o += cout
        out[name] = (W, b)
    return out


def flatten(d):
    parts = []
    for name, _, _, _ in LAYERS:
        W, b = d[name]
        parts += [W.ravel(), b.ravel()]
    return np.concatenate(parts)


def init_params(seed=0):
    """He-normal weights scaled like the reference's small-init convolutions
    (nn_pressure_operator_advanced.py:26-38), zero biases; the padded input and
    output channels are zero."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, cin, cout, _ in LAYERS:
        fan_in = 9 * (FEATURES if name == "e0a" else cin)
        W = rng.standard_normal((3, 3, cin, cout)) * np.sqrt(2.0 / fan_in)
        if name == "e0a":
            W[:, :, FEATURES:, :] = 0.0
        if name == "d0b":
            W *= 0.1
            W[:, :, :, 1:] = 0.0
        d[name] = (W, np.zeros(cout))
    return flatten(d)


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv3x3(X, W, b, emulate_bf16=False):
    """'SAME' 3x3 cross-correlation, zero padding.  X [H][W][Cin]."""
    if emulate_bf16:
        X, W = bf16(X), bf16(W)
    H, Wd, _ = X.shape
    Xp = np.pad(X, ((1, 1), (1, 1), (0, 0)))
    out = np.zeros((H, Wd, W.shape[3])) + b
    for dy in range(3):
        for dx in range(3):
            out += np.einsum("hwc,cd->hwd", Xp[dy:dy + H, dx:dx + Wd], W[dy, dx], optimize=True)
    return out


def conv3x3_backward(X, W, dZ, emulate_bf16=False):
    """Gradients of conv3x3 w.r.t. X, W and b given dZ (pre-activation)."""
    if emulate_bf16:
        Xq, Wq, dZq = bf16(X), bf16(W), bf16(dZ)
    else:
        Xq, Wq, dZq = X, W, dZ
    H, Wd, _ = X.shape
    Xp = np.pad(Xq, ((1, 1), (1, 1), (0, 0)))
    dW = np.zeros_like(W)
    dXp = np.zeros_like(Xp)
    for dy in range(3):
        for dx in range(3):
            dW[dy, dx] = np.einsum("hwc,hwd->cd", Xp[dy:dy + H, dx:dx + Wd], dZq, optimize=True)
            dXp[dy:dy + H, dx:dx + Wd] += np.einsum("hwd,cd->hwc", dZq, Wq[dy, dx], optimize=True)
    return dXp[1:-1, 1:-1], dW, dZ.sum(axis=(0, 1))


def pool2(X):
    return 0.25 * (X[0::2, 0::2] + X[1::2, 0::2] + X[0::2, 1::2] + X[1::2, 1::2])


def pool2_backward(dY):
    H, W, C = dY.shape
    dX = np.zeros((2 * H, 2 * W, C))
    for a in (0, 1):
        for c in (0, 1):
            dX[a::2, c::2] = 0.25 * dY
    return dX


def up2(X):
    return X.repeat(2, axis=0).repeat(2, axis=1)


def up2_backward(dY):
    return dY[0::2, 0::2] + dY[1::2, 0::2] + dY[0::2, 1::2] + dY[1::2, 1::2]


def forward(flat, x, emulate_bf16=False, keep=False):
    """x [H][W][16] -> y [H][W][16] (channel 0 is the prediction)."""
    P = unflatten(flat)
    acts = {}

    def layer(name, inp):
        _, _, _, relu = next(l for l in LAYERS if l[0] == name)
        W, b = P[name]
        z = conv3x3(inp, W, b, emulate_bf16)
        y = np.maximum(z, 0.0) if relu else z
        acts[name] = (inp, y)
        return y

    s0 = layer("e0b", layer("e0a", x))
    s1 = layer("e1b", layer("e1a", pool2(s0)))
    s2 = layer("e2b", layer("e2a", pool2(s1)))
    bott = layer("e3b", layer("e3a", pool2(s2)))
    d2 = layer("d2", up2(bott) + s2)
    d1 = layer("d1", up2(d2) + s1)
    y = layer("d0b", layer("d0a", up2(d1) + s0))
    return (y, acts) if keep else y


def backward(flat, x, dy, emulate_bf16=False):
    """Gradient of sum(dy * forward(x)) w.r.t. the flat parameters."""
    P = unflatten(flat)
    _, acts = forward(flat, x, emulate_bf16, keep=True)
    grads = {}

    def back(name, dout):
        _, _, _, relu = next(l for l in LAYERS if l[0] == name)
        inp, y = acts[name]
        dz = dout * (y > 0) if relu else dout
        dX, dW, db = conv3x3_backward(inp, P[name][0], dz, emulate_bf16)
        grads[name] = (dW, db)
        return dX

    g = back("d0a", back("d0b", dy))            # into up2(d1) + s0
    ds0 = g.copy()
    g = back("d1", up2_backward(g))            # into up2(d2) + s1
    ds1 = g.copy()
    g = back("d2", up2_backward(g))            # into up2(bott) + s2
    ds2 = g.copy()
    g = back("e3a", back("e3b", up2_backward(g)))
    ds2 = ds2 + pool2_backward(g)
    g = back("e2a", back("e2b", ds2))
    ds1 = ds1 + pool2_backward(g)
    g = back("e1a", back("e1b", ds1))
    ds0 = ds0 + pool2_backward(g)
    back("e0a", back("e0b", ds0))
    return flatten(grads)


def mse_loss(y, target):
    """Loss on output channel 0 and its gradient w.r.t. y (all channels)."""
    d = y[..., 0] - target
    loss = np.mean(d * d)
    dy = np.zeros_like(y)
    dy[..., 0] = 2.0 * d / d.size
    return loss, dy


def adam_step(w, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8, clip=1.0):
    """Adam with element-wise gradient clipping to [-clip, clip]
    (training_utils.py:185); t is the 1-based step."""
    g = np.clip(g, -clip, clip)
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return w - lr * mh / (np.sqrt(vh) + eps), m, v


def features(b, mask, p_prev, dx, dy, F, p_true=None):
    """Network input and training target of one pressure solve, on the grid F
    times coarser (the dataset contract of training_utils.py:35-51: the solve's
    right-hand side, the mask and a pressure).  Channel 0: F x F average of the
    residual b - A p_prev of the reference operator (edge ghosts, outlet row
    pinned), channel 1: average mask, channel 2: average p_prev; channels 0 and
    2 divided by their RMS over the grid (per-sample normalisation,
    nn_pressure_operator_advanced.py:56-59).  Target: F x F average of
    p_true - p_prev divided by rms_r * min(lx, ly)^2 / 10.
    Returns (x [h][w][3], target [h][w] or None, out_scale)."""
    b = np.asarray(b, np.float64)
    p = np.asarray(p_prev, np.float64)
    nx, ny = b.shape
    pe = np.pad(p, 1, mode="edge")
    lap = ((pe[2:, 1:-1] - 2 * p + pe[:-2, 1:-1]) / dx ** 2
           + (pe[1:-1, 2:] - 2 * p + pe[1:-1, :-2]) / dy ** 2)
    r = b - lap
    r[-1, :] = 0.0
    h, w = nx // F, ny // F

    def avg(a):
        return a.reshape(h, F, w, F).mean(axis=(1, 3))

    x = np.stack([avg(r), avg(np.asarray(mask, np.float64)), avg(p)], axis=-1)
    rr = max(np.sqrt(np.mean(x[..., 0] ** 2)), 1e-30)
    rp = max(np.sqrt(np.mean(x[..., 2] ** 2)), 1e-30)
    x[..., 0] /= rr
    x[..., 2] /= rp
    lmin = min(nx * dx, ny * dy)
    scale = rr * lmin * lmin / 10.0
    tgt = None if p_true is None else avg(np.asarray(p_true, np.float64) - p) / scale
    return x, tgt, scale


def apply_correction(y0, p_prev, F, scale):
    """p_init = p_prev + bilinear prolongation (cell-centred, clamped at the
    edges) of the prediction y0 [h][w] times scale; the outlet row is 0."""
    p = np.asarray(p_prev, np.float64)
    nx, ny = p.shape
    h, w = y0.shape
    xi = (np.arange(nx) + 0.5) / F - 0.5
    xj = (np.arange(ny) + 0.5) / F - 0.5
    i0 = np.floor(xi).astype(int)
    j0 = np.floor(xj).astype(int)
    ti, tj = (xi - i0)[:, None], (xj - j0)[None, :]
    i1, j1 = np.clip(i0 + 1, 0, h - 1), np.clip(j0 + 1, 0, w - 1)
    i0, j0 = np.clip(i0, 0, h - 1), np.clip(j0, 0, w - 1)
    v = ((1 - ti) * ((1 - tj) * y0[i0][:, j0] + tj * y0[i0][:, j1])
         + ti * ((1 - tj) * y0[i1][:, j0] + tj * y0[i1][:, j1]))
    out = p + v * scale
    out[-1, :] = 0.0
    return out
