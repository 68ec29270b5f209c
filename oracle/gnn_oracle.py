"""CPU oracle of the learned preconditioner's network -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the message-passing network the GPU kernels implement
(svfsiplus_gb300/csrc/k_gnn.cu), forward and backward, used to check the GPU loss and
gradients.  Inputs per node: the residual r / s_r, the prior p / s_p (zero without a
prior) and 4 static features; the output out is the correction scaled by s_o
(s_p with a prior, s_r without): M(r, p) = p + s_o * out.  It reproduces the GPU's storage precisions: weights rounded to BF16,
activations h stored in BF16, the neighbour mean m rounded to BF16 before the dense
layer (the GPU multiplies BF16 tiles on the tensor cores) and for the weight gradient;
arithmetic is FP64 here (FP32 accumulation on the GPU).
"""
from __future__ import annotations

import numpy as np

H, NIN = 64, 12
LAYER = 2 * H * H + H
OFF_W0, OFF_B0 = 0, NIN * H


def off_w(l):
    return OFF_B0 + H + (l - 1) * LAYER


def off_b(l):
    return off_w(l) + 2 * H * H


OFF_WD = OFF_B0 + H + 3 * LAYER
OFF_BD = OFF_WD + H * 4
NPARAM = OFF_BD + 4


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def unpack(p):
    pb = bf16(p)
    W0 = pb[OFF_W0:OFF_W0 + NIN * H].reshape(NIN, H)
    b0 = pb[OFF_B0:OFF_B0 + H]
    Ws = [pb[off_w(l):off_w(l) + 2 * H * H].reshape(2 * H, H) for l in (1, 2, 3)]
    bs = [pb[off_b(l):off_b(l) + H] for l in (1, 2, 3)]
    Wd = pb[OFF_WD:OFF_WD + H * 4].reshape(H, 4)
    bd = pb[OFF_BD:OFF_BD + 4]
    return W0, b0, Ws, bs, Wd, bd


def _mean_gather(rowPtr, colPtr, h):
    deg = np.diff(rowPtr).astype(np.float64)
    rows = np.repeat(np.arange(rowPtr.size - 1), np.diff(rowPtr))
    s = np.zeros_like(h)
    np.add.at(s, rows, h[colPtr])
    return s / deg[:, None], deg


def scales(r, prior):
    """(s_r, s_p or None, s_o) of a residual and an optional prior (both as stored)."""
    n = r.size
    sr = np.sqrt(np.sum(np.asarray(r, np.float64) ** 2) / n)
    sr = sr if sr > 0 else 1.0
    if prior is None:
        return sr, None, sr
    sp = np.sqrt(np.sum(np.asarray(prior, np.float32).astype(np.float64) ** 2) / n)
    return (sr, sp, sp) if sp > 0 else (sr, None, sr)


def forward(p, rowPtr, colPtr, r, stat, prior=None):
    """r (nNo,4) FP64 input; prior (nNo,4) or None; stat (nNo,4).
    Returns (out_raw (nNo,4), output scale s_o, cache)."""
    W0, b0, Ws, bs, Wd, bd = unpack(p)
    sr, sp, so = scales(r, prior)
    pin = np.zeros_like(np.asarray(r, np.float64)) if sp is None else \
        np.asarray(prior, np.float32).astype(np.float64) / sp
    x = np.concatenate([np.asarray(r, np.float32).astype(np.float64) / sr, pin, stat.astype(np.float64)], axis=1)
    z0 = x @ W0 + b0
    h = [bf16(np.maximum(z0, 0.0))]
    masks = [z0 > 0]
    ms = [None]
    for l in range(3):
        m, _ = _mean_gather(rowPtr, colPtr, h[-1])
        mb = bf16(m)  # the neighbour mean enters the dense layer (tensor cores) in BF16
        z = np.concatenate([h[-1], mb], axis=1) @ Ws[l] + bs[l]
        masks.append(z > 0)
        ms.append(mb)
        h.append(bf16(h[-1] + np.maximum(z, 0.0)))
    out = h[3] @ Wd + bd
    return out, so, dict(x=x, h=h, ms=ms, masks=masks)


def loss_grad(p, rowPtr, colPtr, r, xt, stat, prior=None):
    """Relative squared error sum|out - t|^2 / sum|xt / s_o|^2 with t = (xt - prior) / s_o,
    and its gradient."""
    W0, b0, Ws, bs, Wd, bd = unpack(p)
    out, s, c = forward(p, rowPtr, colPtr, r, stat, prior)
    xs = np.asarray(xt, np.float32).astype(np.float64)
    t = xs
    if prior is not None and scales(r, prior)[1] is not None:
        t = t - np.asarray(prior, np.float32).astype(np.float64)
    t = t / s
    E = np.sum((xs / s) ** 2)
    loss = np.sum((out - t) ** 2) / E
    dout = 2.0 * (out - t) / E
    g = np.zeros(NPARAM)
    g[OFF_WD:OFF_WD + H * 4] = (c["h"][3].T @ dout).ravel()
    g[OFF_BD:OFF_BD + 4] = dout.sum(axis=0)
    dh = dout @ Wd.T
    deg = np.diff(rowPtr).astype(np.float64)
    rows = np.repeat(np.arange(rowPtr.size - 1), np.diff(rowPtr))
    for l in (3, 2, 1):
        dz = dh * c["masks"][l]
        X = np.concatenate([c["h"][l - 1], c["ms"][l]], axis=1)
        g[off_w(l):off_w(l) + 2 * H * H] = (X.T @ dz).ravel()
        g[off_b(l):off_b(l) + H] = dz.sum(axis=0)
        dX = dz @ Ws[l - 1].T
        dhd = dh + dX[:, :H]
        dms = dX[:, H:] / deg[:, None]
        prev = dhd.copy()
        np.add.at(prev, rows, dms[colPtr])  # symmetric pattern: sum over neighbours j of dms_j
        dh = prev
    dz0 = dh * c["masks"][0]
    g[OFF_W0:OFF_W0 + NIN * H] = (c["x"].T @ dz0).ravel()
    g[OFF_B0:OFF_B0 + H] = dz0.sum(axis=0)
    return loss, g
