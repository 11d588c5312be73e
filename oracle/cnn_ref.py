"""CPU restatement of the learned-guess network, used only to check the GPU kernels.

TEST INFRASTRUCTURE: imported by tests/ and nothing else.  The reference has no such network
(its CG of common/field.f90:319-461 starts from the previous step's dB), so this file is the
definition the CUDA kernels are checked against, not a restatement of reference code; its
backward pass is pinned by finite differences in tests/test_cnn_oracle.py.

Network: six periodic 3x3 convolutions, channels (padded) 16 -> 48 -> 48 -> 48 -> 48 -> 48 -> 8,
GELU (erf form) after the first five; weights [9][cout][cin] with tap = (dy+1)*3 + (dx+1):
    out[n, y, x, co] = b[co] + sum_{tap, ci} w[tap, co, ci] * in[n, (y+dy) % H, (x+dx) % W, ci].
With bf16=True every tensor the GPU keeps in BF16 (inputs, weights, activations, stored
pre-activations, pre-activation gradients) is rounded to BF16 (round to nearest even) where the
GPU rounds it; sums are exact (float64).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

LAYERS = ((16, 48), (48, 48), (48, 48), (48, 48), (48, 48), (48, 8))  # (cin, cout), padded
NREAL_IN, NREAL_OUT = 9, 3
GRAD_CH = 16  # channels of the output gradient


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even); returns float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def _shift(x, dy, dx):
    """s[n, y, x] = x[n, (y+dy) % H, (x+dx) % W]."""
    return np.roll(x, shift=(-dy, -dx), axis=(1, 2))


def conv(x, w, b=None):
    out = np.zeros(x.shape[:3] + (w.shape[1],))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        out += _shift(x, dy, dx) @ w[tap].T
    if b is not None:
        out += b
    return out


def conv_input_grad(dout, w):
    """d(in) of conv for the output gradient dout: sum_tap W_tap^T dout[(y-dy), (x-dx)]."""
    din = np.zeros(dout.shape[:3] + (w.shape[2],))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        din += _shift(dout, -dy, -dx) @ w[tap]
    return din


def conv_weight_grad(x, dz):
    dw = np.zeros((9, dz.shape[3], x.shape[3]))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        dw[tap] = np.einsum("nyxc,nyxd->cd", dz, _shift(x, dy, dx))
    return dw, dz.sum(axis=(0, 1, 2))


def init_params(seed: int = 0, scale: float = 1.0):
    """He-style initial weights, zero on the padded channels; biases zero."""
    rng = np.random.Generator(np.random.Philox(seed))
    params = []
    for l, (cin, cout) in enumerate(LAYERS):
        rin = NREAL_IN if l == 0 else cin
        rout = NREAL_OUT if l == len(LAYERS) - 1 else cout
        w = np.zeros((9, cout, cin))
        std = scale * np.sqrt(2.0 / (9 * rin))
        w[:, :rout, :rin] = std * rng.standard_normal((9, rout, rin))
        params.append((w.astype(np.float32).astype(np.float64), np.zeros(cout)))
    return params


def flatten(params) -> np.ndarray:
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in params]).astype(np.float32)


def unflatten(flat) -> list:
    flat = np.asarray(flat, dtype=np.float64)
    out, o = [], 0
    for cin, cout in LAYERS:
        n = 9 * cout * cin
        out.append((flat[o:o + n].reshape(9, cout, cin), flat[o + n:o + n + cout].copy()))
        o += n + cout
    return out


def nparams() -> int:
    return sum(9 * ci * co + co for ci, co in LAYERS)


def forward(x, params, bf=True):
    """x: [n][H][W][16].  Returns (pred [n][H][W][8], cache)."""
    r = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    a = r(x)
    acts, zs = [a], []
    for l, (w, b) in enumerate(params):
        z = conv(a, r(w), b)
        if l == len(params) - 1:
            return z, (acts, zs)
        zs.append(r(z))
        a = r(gelu(z))
        acts.append(a)


def loss_and_grad(pred, target):
    """0.5 * mean over pixels and the 3 outputs of (pred - target)^2, and d/dpred as [..][16]."""
    e = pred[..., :NREAL_OUT] - target
    count = e.size
    g = np.zeros(pred.shape[:3] + (GRAD_CH,))
    g[..., :NREAL_OUT] = e / count
    return 0.5 * float(np.sum(e * e)) / count, g


def backward(cache, dpred, params, bf=True):
    """Parameter gradients [(dw, db)] for the output gradient dpred [..][16]."""
    r = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    acts, zs = cache
    grads = [None] * len(params)
    dz = r(dpred)
    for l in range(len(params) - 1, -1, -1):
        w, b = params[l]
        cout = w.shape[1]
        dw, db = conv_weight_grad(acts[l], dz[..., :cout])
        grads[l] = (dw, db)
        if l == 0:
            break
        wpad = np.zeros((9, dz.shape[3], w.shape[2]))
        wpad[:, :cout, :] = r(w)
        da = conv_input_grad(dz, wpad)
        dz = r(da * gelu_grad(zs[l - 1]))
    return grads
