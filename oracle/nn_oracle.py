"""Test infrastructure: numpy restatement (FP64 arithmetic) of the field
surrogate's layers (hpsim_gb300/csrc/nn.cu) -- the oracle their forward
values and gradients are tested against.  Never used by the library.

Layouts as the kernels: tensors [batch][channel][z][r], weights
[c_out][c_in][3][3]; a layer upsamples its input by `up` (nearest), pads by
one and applies a 3x3 convolution with stride `stride`, then bias and ReLU.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """Round float32 values to BF16 (nearest, ties to even) and back."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def _upsample(x, up):
    return x if up == 1 else x.repeat(up, axis=2).repeat(up, axis=3)


def _windows(x, stride):
    """[B, C, Ho, Wo, 3, 3] windows of the zero-padded input."""
    B, Ci, H, W = x.shape
    Ho, Wo = (H - 1) // stride + 1, (W - 1) // stride + 1
    xp = np.zeros((B, Ci, H + 2, W + 2), x.dtype)
    xp[:, :, 1:-1, 1:-1] = x
    out = np.empty((B, Ci, Ho, Wo, 3, 3), x.dtype)
    for ky in range(3):
        for kx in range(3):
            out[..., ky, kx] = xp[:, :, ky:ky + stride * (Ho - 1) + 1:stride, kx:kx + stride * (Wo - 1) + 1:stride]
    return out


def conv_forward(x, w, b, stride, up, relu):
    """FP64 pre-activation and activation of one layer."""
    xu = _upsample(np.asarray(x, np.float64), up)
    win = _windows(xu, stride)
    z = np.einsum("bchwij,ocij->bohw", win, np.asarray(w, np.float64)) + np.asarray(b, np.float64)[None, :, None, None]
    return z, (np.maximum(z, 0.0) if relu else z)


def conv_backward(x, w, y, relu, dy, stride, up):
    """dz (dy masked by y > 0), dx, dw, db of one layer, FP64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    dz = np.where(np.asarray(y, np.float64) > 0.0, dy, 0.0) if relu else np.asarray(dy, np.float64)
    xu = _upsample(x, up)
    win = _windows(xu, stride)
    dw = np.einsum("bohw,bchwij->ocij", dz, win)
    db = dz.sum(axis=(0, 2, 3))
    # dx: scatter dz through the windows, then sum the upsampled copies
    B, Ci, Hu, Wu = xu.shape
    dxp = np.zeros((B, Ci, Hu + 2, Wu + 2))
    Ho, Wo = dz.shape[2], dz.shape[3]
    contrib = np.einsum("bohw,ocij->bchwij", dz, w)
    for ky in range(3):
        for kx in range(3):
            dxp[:, :, ky:ky + stride * (Ho - 1) + 1:stride, kx:kx + stride * (Wo - 1) + 1:stride] += contrib[..., ky, kx]
    dxu = dxp[:, :, 1:-1, 1:-1]
    H, W = x.shape[2], x.shape[3]
    dx = dxu.reshape(B, Ci, H, up, W, up).sum(axis=(3, 5))
    return dz, dx, dw, db


def gmean_forward(y):
    y = np.asarray(y, np.float64)
    return y + y.mean(axis=(2, 3), keepdims=True)


def gmean_backward(d):
    d = np.asarray(d, np.float64)
    return d + d.mean(axis=(2, 3), keepdims=True)


def net_forward(x, ws, bs, arch, gmean_after, skip):
    """Whole-network forward in FP64, composed as the surrogate does:
    layer l reads the previous layer's output; the output of layer
    `gmean_after` gets its plane mean added; layer l in `skip` adds the output
    of layer skip[l] to its activation.  Returns (ins, acts, outs)."""
    ins, acts, outs = [], [], []
    cur = np.asarray(x, np.float64)
    for l, (ci, co, stride, up, relu) in enumerate(arch):
        _, y = conv_forward(cur, ws[l], bs[l], stride, up, relu)
        ins.append(cur)
        acts.append(y)
        out = y
        if l == gmean_after:
            out = gmean_forward(y)
        if l in skip:
            out = y + outs[skip[l]]
        outs.append(out)
        cur = out
    return ins, acts, outs


def net_backward(fwd, ws, arch, gmean_after, skip, dout):
    """Gradients (dws, dbs) of sum(dout * prediction) through net_forward."""
    ins, acts, _ = fwd
    n = len(arch)
    g = [None] * n
    g[-1] = np.asarray(dout, np.float64)
    dws, dbs = [None] * n, [None] * n
    for l in reversed(range(n)):
        gl = g[l]
        if l in skip:
            s = skip[l]
            g[s] = gl if g[s] is None else g[s] + gl
        if l == gmean_after:
            gl = gmean_backward(gl)
        ci, co, stride, up, relu = arch[l]
        _, dx, dw, db = conv_backward(ins[l], ws[l], acts[l], relu, gl, stride, up)
        dws[l], dbs[l] = dw, db
        if l > 0:
            g[l - 1] = dx if g[l - 1] is None else g[l - 1] + dx
    return dws, dbs
