"""Double-precision restatement of the radiance cache -- the ORACLE of its
encoding, forward pass, relative-L2 loss and gradients.  TEST
INFRASTRUCTURE ONLY (the product path is the CUDA library).

Follows the published methods the library's kernels implement (multiresolution
hash encoding of Mueller et al. 2022, real spherical harmonics of degree < 4,
a bias-free ReLU MLP): the hash-grid cell lookup is done in float32 exactly
as the kernel does it (so both pick the same table entries); everything after
that is float64.  The weights and table values fed in are rounded to the
precisions the kernel reads (BF16 weights, FP16 table) when `emulate=True`.
"""
from __future__ import annotations

import math

import numpy as np

LEVELS = 16
W = 64
HIDDEN = 5
OUT = 16
NPARAM = (HIDDEN * W + OUT) * W


def levels(T: int, base: int, maxres: int):
    b = math.exp((math.log(maxres) - math.log(base)) / (LEVELS - 1))
    res, dense = [], []
    for l in range(LEVELS):
        r = math.floor(base * b ** l + 1e-6)
        res.append(float(r))
        st = r + 1
        dense.append(st if st ** 3 <= T else 0)
    return res, dense


def bf16_round(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def sh16(d):
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return np.stack([
        np.full_like(x, 0.28209479177387814), -0.48860251190291987 * y, 0.48860251190291987 * z,
        -0.48860251190291987 * x, 1.0925484305920792 * x * y, -1.0925484305920792 * y * z,
        0.94617469575756008 * zz - 0.31539156525252005, -1.0925484305920792 * x * z,
        0.54627421529603959 * (xx - yy), 0.59004358992664352 * y * (-3.0 * xx + yy), 2.8906114426405538 * x * y * z,
        0.45704579946446572 * y * (1.0 - 5.0 * zz), 0.3731763325901154 * z * (5.0 * zz - 3.0),
        0.45704579946446572 * x * (1.0 - 5.0 * zz), 1.4453057213202769 * z * (xx - yy),
        0.59004358992664352 * x * (-xx + 3.0 * yy)], axis=1)


class Cache:
    def __init__(self, T, aabb_min, aabb_max, base=16, maxres=2048):
        self.T = T
        self.res, self.dense = levels(T, base, maxres)
        self.lo = np.asarray(aabb_min, np.float32)
        hi = np.asarray(aabb_max, np.float32)
        self.s = (np.float32(1.0) / (hi - self.lo)).astype(np.float32)

    def cells(self, pos, l):
        """Corner coordinates and fractions of level l (float32, as the kernel)."""
        x = np.clip((pos.astype(np.float32) - self.lo) * self.s, np.float32(0.0), np.float32(0.999999)).astype(np.float32)
        p = (x * np.float32(self.res[l])).astype(np.float32)
        c = np.floor(p)
        f = (p - c).astype(np.float64)
        return c.astype(np.uint64), f

    def index(self, l, x, y, z):
        st = self.dense[l]
        if st:
            return (x + y * st + z * st * st).astype(np.int64)
        h = (x.astype(np.uint64) ^ ((y.astype(np.uint64) * 2654435761) & 0xFFFFFFFF)
             ^ ((z.astype(np.uint64) * 805459861) & 0xFFFFFFFF)) & 0xFFFFFFFF
        return (h & (self.T - 1)).astype(np.int64)

    def corners(self, pos, l):
        c, f = self.cells(pos, l)
        out = []
        for k in range(8):
            dx, dy, dz = k & 1, (k >> 1) & 1, k >> 2
            w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
            out.append((self.index(l, c[:, 0] + dx, c[:, 1] + dy, c[:, 2] + dz), w))
        return out

    def encode(self, table, rec):
        """table: (LEVELS, T, 2) float64; rec: (n, 16) records -> X (n, 64)."""
        n = len(rec)
        X = np.zeros((n, 64))
        pos = rec[:, 0:3]
        for l in range(LEVELS):
            for idx, w in self.corners(pos, l):
                X[:, 2 * l:2 * l + 2] += w[:, None] * table[l, idx]
        X[:, 32:48] = sh16(rec[:, 4:7].astype(np.float64))
        X[:, 48:51] = rec[:, 8:11]
        X[:, 51] = rec[:, 3]
        X[:, 52] = rec[:, 11]
        return X

    def forward(self, mlp, table, rec, bf16=False):
        """bf16=True rounds the input and every activation to BF16, as the
        kernel stores them."""
        q = bf16_round if bf16 else (lambda x: x)
        Ws = [mlp[l * W * W:(l + 1) * W * W].reshape(W, W) for l in range(HIDDEN)]
        Wo = mlp[HIDDEN * W * W:].reshape(OUT, W)
        A = [q(self.encode(table, rec))]
        for Wl in Ws:
            A.append(q(np.maximum(A[-1] @ Wl.T, 0.0)))
        P = A[-1] @ Wo.T
        return A, P

    def loss_and_grads(self, mlp, table, rec, bf16=False):
        """bf16=True also rounds the backward deltas to BF16 (the kernel keeps
        them in BF16 shared-memory tiles)."""
        q = bf16_round if bf16 else (lambda x: x)
        n = len(rec)
        Ws = [mlp[l * W * W:(l + 1) * W * W].reshape(W, W) for l in range(HIDDEN)]
        Wo = mlp[HIDDEN * W * W:].reshape(OUT, W)
        A, P = self.forward(mlp, table, rec, bf16)
        t = rec[:, 12:15].astype(np.float64)
        p = P[:, :3]
        den = p * p + 0.01
        loss = np.sum((p - t) ** 2 / den) / (3 * n)
        dP = np.zeros_like(P)
        dP[:, :3] = 2.0 * (p - t) / den / (3 * n)
        dP = q(dP)
        gW = [None] * (HIDDEN + 1)
        gW[HIDDEN] = dP.T @ A[HIDDEN]
        dA = q(dP @ Wo)
        for l in range(HIDDEN - 1, -1, -1):
            dZ = dA * (A[l + 1] > 0)
            gW[l] = dZ.T @ A[l]
            dA = q(dZ @ Ws[l])
        gmlp = np.concatenate([g.reshape(-1) for g in gW])
        ggrid = np.zeros((LEVELS, self.T, 2))
        pos = rec[:, 0:3]
        for l in range(LEVELS):
            g = dA[:, 2 * l:2 * l + 2]
            for idx, w in self.corners(pos, l):
                np.add.at(ggrid[l], idx, w[:, None] * g)
        return loss, gmlp, ggrid.reshape(-1), P


def emulate_params(mlp, grid):
    """The values the kernel reads: BF16 weights, FP16 table."""
    return bf16_round(mlp), np.asarray(grid, np.float32).astype(np.float16).astype(np.float64)
