"""CPU float64 restatement of the learned distance bound -- test infrastructure only.

Nothing in the product imports this module: the GPU tests compare the library's
tg_surrogate_* kernels against it.  It restates, in numpy:

* the multiresolution hash-grid encoding of Mueller, Evans, Schied and Keller, "Instant
  Neural Graphics Primitives with a Multiresolution Hash Encoding" (SIGGRAPH 2022),
  section 3: level l has Res[l] cells per axis over the domain box; a point's 8 cell
  corners index the level's table densely while (Res + 1)^3 fits it, else by the paper's
  hash (x * 1) xor (y * 2654435761) xor (z * 805459861) mod T; features are the trilinear
  blend of the corners' two values.  Corner selection and weights are computed in float32
  exactly as the kernels do (the cell index must agree bit for bit); the blend is float64.
* the 32 -> 64 -> 64 -> 64 -> 1 ReLU network with the kernels' BF16 roundings at the same
  places (inputs, hidden activations, the backward pass's dZ, all weights) and float64
  everywhere the kernels accumulate in FP32;
* the mean-squared-error gradient against clamp(d, -clamp, clamp) and the Adam update
  (Kingma and Ba 2015) with bias correction.

There is no reference implementation of this part: Tangerine has no learned component.
"""

from __future__ import annotations

import numpy as np

LEVELS = 16
W1, B1, W2, B2, W3, B3, W4, B4, PARAMS = 0, 2048, 2112, 6208, 6272, 10368, 10432, 10496, 10497


def bf16(x) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) through float32; returned as float64."""
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    bits = x32.view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return rounded.view(np.float32).astype(np.float64)


class Grid:
    """Encoding geometry, as tg_surrogate_get_info reports it."""

    def __init__(self, resolutions, dense_levels, table_size, lo=(-2, -2, -2), hi=(2, 2, 2), clamp=0.5):
        self.res = [int(r) for r in resolutions]
        self.dense = int(dense_levels)
        self.T = int(table_size)
        self.lo = np.asarray(lo, np.float32)
        self.scale = (np.float32(1.0) / (np.asarray(hi, np.float32) - self.lo)).astype(np.float32)
        self.clamp = float(clamp)

    @classmethod
    def from_info(cls, info, lo=(-2, -2, -2), hi=(2, 2, 2), clamp=0.5):
        return cls(list(info.resolutions), info.dense_levels, info.table_size, lo, hi, clamp)

    def unit(self, points):
        p = np.asarray(points, np.float32).reshape(-1, 3)
        u = (p - self.lo) * self.scale
        return np.clip(u, np.float32(0), np.float32(1)).astype(np.float32)

    def corners(self, u, level):
        """(index (n, 8) int64, weight (n, 8) float64) of the level's cell corners."""
        R = self.res[level]
        x = u * np.float32(R)
        c = np.clip(np.floor(x).astype(np.int64), 0, R - 1)
        f = (x - c.astype(np.float32)).astype(np.float32)
        idx = np.empty((u.shape[0], 8), np.int64)
        w = np.empty((u.shape[0], 8), np.float64)
        one = np.float32(1)
        for k in range(8):
            d = np.array([k & 1, (k >> 1) & 1, k >> 2])
            cx, cy, cz = (c[:, a] + d[a] for a in range(3))
            if (self.dense >> level) & 1:
                s = R + 1
                idx[:, k] = cx + s * (cy + s * cz)
            else:
                h = (cx.astype(np.uint32) ^ (cy.astype(np.uint32) * np.uint32(2654435761))
                     ^ (cz.astype(np.uint32) * np.uint32(805459861)))
                idx[:, k] = (h & np.uint32(self.T - 1)).astype(np.int64)
            wx = f[:, 0] if d[0] else one - f[:, 0]
            wy = f[:, 1] if d[1] else one - f[:, 1]
            wz = f[:, 2] if d[2] else one - f[:, 2]
            w[:, k] = ((wx * wy).astype(np.float32) * wz).astype(np.float32)
        return idx, w

    def encode(self, table, points):
        t = np.asarray(table, np.float64).reshape(LEVELS, self.T, 2)
        u = self.unit(points)
        feat = np.empty((u.shape[0], 2 * LEVELS))
        for l in range(LEVELS):
            idx, w = self.corners(u, l)
            feat[:, 2 * l:2 * l + 2] = np.einsum("nk,nkf->nf", w, t[l][idx])
        return feat


def _exact(x):
    return np.asarray(x, np.float64)


def _unpack(mlp, r):
    m = np.asarray(mlp, np.float64)
    return (r(m[W1:B1]).reshape(64, 32), m[B1:W2], r(m[W2:B2]).reshape(64, 64), m[B2:W3],
            r(m[W3:B3]).reshape(64, 64), m[B3:W4], r(m[W4:B4]), m[B4])


def forward(grid: Grid, table, mlp, points, rounded=True):
    """Activations and output of the network at the points (rounded=False: no BF16
    rounding anywhere, for checking the formulas against finite differences)."""
    r = bf16 if rounded else _exact
    w1, b1, w2, b2, w3, b3, w4, b4 = _unpack(mlp, r)
    x = r(grid.encode(table, points))
    z1 = x @ w1.T + b1
    h1 = r(np.maximum(z1, 0))
    z2 = h1 @ w2.T + b2
    h2 = r(np.maximum(z2, 0))
    z3 = h2 @ w3.T + b3
    h3 = np.maximum(z3, 0)
    s = h3 @ w4 + b4
    return dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, s=s)


def gradients(grid: Grid, table, mlp, samples, rounded=True):
    """(table_grad, mlp_grad, summed squared error) of the mean squared error against
    clamp(d) over the samples (x, y, z, d)."""
    r = bf16 if rounded else _exact
    smp = np.asarray(samples, np.float32).reshape(-1, 4)
    n = smp.shape[0]
    w1, b1, w2, b2, w3, b3, w4, b4 = _unpack(mlp, r)
    a = forward(grid, table, mlp, smp[:, :3], rounded)
    t = np.clip(smp[:, 3].astype(np.float64), -grid.clamp, grid.clamp)
    diff = a["s"] - t
    g = 2.0 * diff / n
    gm = np.zeros(PARAMS)
    gm[W4:B4] = g @ a["h3"]
    gm[B4] = g.sum()
    dz3 = r(g[:, None] * w4[None, :] * (a["z3"] > 0))
    dz2 = r((dz3 @ w3) * (a["z2"] > 0))
    gm[W3:B3] = (dz3.T @ a["h2"]).ravel()
    gm[B3:W4] = dz3.sum(0)
    dz1 = r((dz2 @ w2) * (a["z1"] > 0))
    gm[W2:B2] = (dz2.T @ a["h1"]).ravel()
    gm[B2:W3] = dz2.sum(0)
    dx = dz1 @ w1
    gm[W1:B1] = (dz1.T @ a["x"]).ravel()
    gm[B1:W2] = dz1.sum(0)
    gt = np.zeros((LEVELS, grid.T, 2))
    u = grid.unit(smp[:, :3])
    for l in range(LEVELS):
        idx, w = grid.corners(u, l)
        for k in range(8):
            np.add.at(gt[l], idx[:, k], w[:, k:k + 1] * dx[:, 2 * l:2 * l + 2])
    return gt.ravel(), gm, float(np.sum(diff * diff))


def adam(params, grads, m, v, step, rate, beta1=0.9, beta2=0.99, eps=1e-15):
    """One Adam update (returns new params, m, v); `step` counts from 1."""
    p = np.asarray(params, np.float64)
    g = np.asarray(grads, np.float64)
    m = beta1 * np.asarray(m, np.float64) + (1 - beta1) * g
    v = beta2 * np.asarray(v, np.float64) + (1 - beta2) * g * g
    p = p - rate * (m / (1 - beta1 ** step)) / (np.sqrt(v / (1 - beta2 ** step)) + eps)
    return p, m, v
