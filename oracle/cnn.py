"""CPU FP64 restatement of the learned preconditioner's network.  TEST
INFRASTRUCTURE ONLY: the GPU kernels (maple3dmt_gb300/csrc/cuda/learned.cu)
are checked against it; nothing in the product imports it.

The network: `n_layers` 3x3x3 convolutions with zero padding ("same" size)
on a dense grid [D, H, W] with channels last, ReLU after every layer but the
last, biases in every layer.  Weights w[l] have shape [27, c_out, c_in] with
tap t = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1).  The reference has no learned
component; this restatement is the checker the gradient tests use.
"""
from __future__ import annotations

import numpy as np

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _shift(x, dz, dy, dx):
    """y[z, y, x] = x[z + dz, y + dy, x + dx] (zero outside), channels last."""
    D, H, W = x.shape[:3]
    out = np.zeros_like(x)
    zs, ys, xs = slice(max(0, -dz), D - max(0, dz)), slice(max(0, -dy), H - max(0, dy)), slice(max(0, -dx),
                                                                                            W - max(0, dx))
    zd, yd, xd = slice(max(0, dz), D - max(0, -dz)), slice(max(0, dy), H - max(0, -dy)), slice(max(0, dx),
                                                                                            W - max(0, -dx))
    out[zs, ys, xs] = x[zd, yd, xd]
    return out


def conv3d(x, w, b):
    """x [D, H, W, c_in], w [27, c_out, c_in], b [c_out] -> [D, H, W, c_out]."""
    y = np.zeros(x.shape[:3] + (w.shape[1],), dtype=np.float64)
    for t, (dz, dy, dx) in enumerate(TAPS):
        y += _shift(x, dz, dy, dx) @ w[t].T
    return y + b


def conv3d_dgrad(dy, w):
    """Gradient w.r.t. the input of conv3d: dx[v] = sum_t dy[v - off_t] w[t]."""
    dx = np.zeros(dy.shape[:3] + (w.shape[2],), dtype=np.float64)
    for t, (oz, oy, ox) in enumerate(TAPS):
        dx += _shift(dy, -oz, -oy, -ox) @ w[t]
    return dx


def conv3d_wgrad(x, dy):
    """Gradient w.r.t. the weights: dw[t] = sum_v dy[v]^T x[v + off_t]."""
    c_out, c_in = dy.shape[-1], x.shape[-1]
    dw = np.zeros((27, c_out, c_in))
    dyf = dy.reshape(-1, c_out)
    for t, (dz, ddy, dx) in enumerate(TAPS):
        dw[t] = dyf.T @ _shift(x, dz, ddy, dx).reshape(-1, c_in)
    return dw


def forward(x, ws, bs):
    """Activations of every layer: acts[0] = x, acts[l + 1] = layer l output."""
    acts = [x]
    for l, (w, b) in enumerate(zip(ws, bs)):
        y = conv3d(acts[-1], w, b)
        if l < len(ws) - 1:
            y = np.maximum(y, 0.0)
        acts.append(y)
    return acts


def backward(acts, ws, dout):
    """Weight and bias gradients of sum(dout * network(x)) and d/dx."""
    n = len(ws)
    dws, dbs = [None] * n, [None] * n
    d = dout
    for l in range(n - 1, -1, -1):
        if l < n - 1:
            d = d * (acts[l + 1] > 0)
        dws[l] = conv3d_wgrad(acts[l], d)
        dbs[l] = d.reshape(-1, d.shape[-1]).sum(0)
        d = conv3d_dgrad(d, ws[l])
    return dws, dbs, d


def mse_loss(pred, target):
    """0.5 * mean over samples of |pred - target|^2 / n_voxels; and d/dpred."""
    n = pred.shape[0] * int(np.prod(pred.shape[1:4]))
    diff = pred - target
    return 0.5 * float(np.sum(diff * diff)) / n, diff / n
