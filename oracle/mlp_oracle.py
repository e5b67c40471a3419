"""FP64 numpy restatement of the per-atom features and the charge MLP.

TEST INFRASTRUCTURE ONLY (the checker of tb_mlp_features / tb_mlp_grad /
tb_mlp_predict).  The learned start has no counterpart in the reference; this
file restates the definitions in include/largetb.h in plain numpy:
features = 16 Si + 16 O Gaussian radial sums with a cosine cutoff at 5 A;
y = w3 . silu(W2 silu(W1 x~ + b1) + b2) + b3, weights rounded to BF16
(round-to-nearest-even), loss = mean squared error.
"""
from __future__ import annotations

import numpy as np

BOHR_PER_ANG = 1.88973
NF, NH = 32, 64


def features(xyz, species, box):
    xyz = np.asarray(xyz, float).reshape(-1, 3)
    n = xyz.shape[0]
    box = np.asarray(box, float)
    d = xyz[None, :, :] - xyz[:, None, :]
    for q in range(3):
        if box[q] > 0:
            d[..., q] -= box[q] * np.rint(d[..., q] / box[q])
    r = np.sqrt((d ** 2).sum(-1)) / BOHR_PER_ANG
    np.fill_diagonal(r, np.inf)
    mask = r < 5.0
    rs = np.where(mask, r, 0.0)
    fc = np.where(mask, 0.5 * (np.cos(np.pi * rs / 5.0) + 1.0), 0.0)
    mu = 0.8 + 0.28 * np.arange(16)
    g = np.exp(-12.5 * (rs[..., None] - mu) ** 2) * fc[..., None]
    si = (np.asarray(species) == 14)
    out = np.zeros((n, NF))
    out[:, :16] = g[:, si, :].sum(1)
    out[:, 16:] = g[:, ~si, :].sum(1)
    return out


def bf16(a):
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + NH * NF].reshape(NH, NF); o += NH * NF
    b1 = p[o:o + NH]; o += NH
    W2 = p[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = p[o:o + NH]; o += NH
    w3 = p[o:o + NH]; o += NH
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, norm, feat):
    q = bf16(params)
    W1, b1, W2, b2, w3, b3 = unpack(q)
    mean, istd = np.asarray(norm[:NF], float), np.asarray(norm[NF:], float)
    x = (np.asarray(feat, float) - mean) * istd
    z1 = x @ W1.T + b1
    h1 = silu(z1)
    z2 = h1 @ W2.T + b2
    h2 = silu(z2)
    return h2 @ w3 + b3, (x, z1, h1, z2, h2, W2, w3)


def forward_bf16_inputs(params, norm, feat):
    """forward() with each layer's input rounded to BF16 as well -- the
    numerics of the tensor-core inference kernel (the normalisation in FP32,
    as on the device)."""
    q = bf16(params)
    W1, b1, W2, b2, w3, b3 = unpack(q)
    mean, istd = np.asarray(norm[:NF], np.float32), np.asarray(norm[NF:], np.float32)
    x = bf16((np.asarray(feat, np.float32) - mean) * istd)
    h1 = silu(x @ W1.T + b1)
    z2 = bf16(h1) @ W2.T + b2
    return silu(z2) @ w3 + b3


def grad(params, norm, feat, target):
    y, (x, z1, h1, z2, h2, W2, w3) = forward(params, norm, feat)
    n = y.shape[0]
    dy = 2.0 * (y - target) / n
    gw3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = (dy[:, None] * w3[None, :]) * dsilu(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * dsilu(z1)
    gW1 = dz1.T @ x
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return g, float(((y - target) ** 2).mean())
