"""TEST INFRASTRUCTURE ONLY: CPU FP64 restatement of the closure network.

Reference values for the GPU closure kernels (BF16 tensor-core convolutions): the same
three periodic 3x3x3 convolutions 4 -> 32 -> 32 -> 2 with GELU (tanh form), the same
mean-squared-error loss and its exact gradient, in numpy float64.  The
network has no counterpart in the reference; its definition is the one in
include/lattice.h (lat_net_*).  Optionally the BF16 rounding points of the GPU
path are emulated (inputs, weights, stored activations and gradients), so
the remaining GPU/CPU difference is FP32 accumulation order only.

Flat parameter layout: W1[27][8][32] b1[32] W2[27][32][32] b2[32]
W3[27][32][8] b3[8]; tap = (dz+1)*9 + (dy+1)*3 + (dx+1) for the input offset
(dx, dy, dz).  Activations are channels-last [lattice][z][y][x][C].
"""
from __future__ import annotations

import numpy as np

C_IN, C_HID, C_OUT = 8, 32, 8
SHAPES = [("W1", (27, C_IN, C_HID)), ("b1", (C_HID,)), ("W2", (27, C_HID, C_HID)), ("b2", (C_HID,)),
          ("W3", (27, C_HID, C_OUT)), ("b3", (C_OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)
OFFSETS = [(dz - 1, dy - 1, dx - 1) for dz in range(3) for dy in range(3) for dx in range(3)]


def unflatten(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def flatten(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), via the FP32 bit pattern."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_C = np.sqrt(2.0 / np.pi)


def gelu(z):
    """GELU in its tanh form (the network's activation)."""
    return 0.5 * z * (1.0 + np.tanh(_C * (z + 0.044715 * z ** 3)))


def gelu_d(z):
    t = np.tanh(_C * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3 * 0.044715 * z * z)


def _shift(a, off):
    """a[s + off] on the periodic lattice; a: [B, nz, ny, nx, C]."""
    dz, dy, dx = off
    return np.roll(a, shift=(-dz, -dy, -dx), axis=(1, 2, 3))


def conv(a, W, b=None):
    out = 0.0
    for t, off in enumerate(OFFSETS):
        out = out + _shift(a, off) @ W[t]
    return out if b is None else out + b


def conv_back_data(d, W):
    """Gradient with respect to the input of conv(., W) for output gradient d."""
    out = 0.0
    for t, off in enumerate(OFFSETS):
        out = out + np.roll(d @ W[t].T, shift=off, axis=(1, 2, 3))
    return out


def conv_back_weight(a, d):
    return np.stack([np.einsum("bzyxi,bzyxo->io", _shift(a, off), d) for off in OFFSETS])


def pack_inputs(samples, shift, scale, emulate=False):
    """samples: [B, 6, nz, ny, nx] FP32; returns the padded network input [B, nz, ny, nx, 8]."""
    x = np.zeros(samples.shape[:1] + samples.shape[2:] + (C_IN,))
    for c in range(4):
        v = (samples[:, c].astype(np.float64) - shift[c]) * scale[c]
        x[..., c] = bf16(v) if emulate else v
    return x


def forward(p, x, emulate=False):
    P = unflatten(p)
    Wq = {k: (bf16(v) if emulate and k.startswith("W") else v) for k, v in P.items()}
    z1 = conv(x, Wq["W1"], P["b1"])
    a1 = gelu(z1)
    if emulate:
        a1 = bf16(a1)
    z2 = conv(a1, Wq["W2"], P["b2"])
    a2 = gelu(z2)
    if emulate:
        a2 = bf16(a2)
    out = conv(a2, Wq["W3"], P["b3"])[..., :2]
    return out, (x, z1, a1, z2, a2, Wq)


def loss_and_grad(p, samples, norm, emulate=False):
    """norm = (shift[4], scale[4], out_scale[2]).  Returns (loss, flat gradient)."""
    shift, scale, oscale = norm
    x = pack_inputs(samples, shift, scale, emulate)
    out, (x, z1, a1, z2, a2, Wq) = forward(p, x, emulate)
    tgt = np.stack([samples[:, 4] * oscale[0], samples[:, 5] * oscale[1]], axis=-1).astype(np.float64)
    e = out - tgt
    n = e.size
    loss = float(np.sum(e * e) / n)
    d3 = np.zeros(out.shape[:-1] + (C_OUT,))
    d3[..., :2] = 2.0 * e / n
    if emulate:
        d3 = bf16(d3)
    g = {}
    g["W3"] = conv_back_weight(a2, d3)
    g["b3"] = d3.sum(axis=(0, 1, 2, 3))
    zz2 = bf16(z2) if emulate else z2
    d2 = conv_back_data(d3, Wq["W3"]) * gelu_d(zz2)
    if emulate:
        d2 = bf16(d2)
    g["W2"] = conv_back_weight(a1, d2)
    g["b2"] = d2.sum(axis=(0, 1, 2, 3))
    zz1 = bf16(z1) if emulate else z1
    d1 = conv_back_data(d2, Wq["W2"]) * gelu_d(zz1)
    if emulate:
        d1 = bf16(d1)
    g["W1"] = conv_back_weight(x, d1)
    g["b1"] = d1.sum(axis=(0, 1, 2, 3))
    return loss, flatten(g)


def mask() -> np.ndarray:
    """1 for live parameters, 0 for the padded channels (inputs 4..7, outputs 2..7)."""
    m = {name: np.ones(shp) for name, shp in SHAPES}
    m["W1"][:, 4:, :] = 0.0
    m["W3"][:, :, 2:] = 0.0
    m["b3"][2:] = 0.0
    return flatten(m)
