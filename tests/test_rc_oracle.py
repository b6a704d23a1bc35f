"""The radiance cache's FP64 oracle checked against central finite
differences (the reference engine has no radiance cache, so the oracle's
backward pass is pinned by differentiation instead).  CPU only."""
import numpy as np

import rc_oracle

LO, HI = (0.0, 0.0, 0.0), (10.0, 10.0, 10.0)


def setup(seed=0, n=24, T=2 ** 10):
    rng = np.random.default_rng(seed)
    c = rc_oracle.Cache(T, LO, HI, base=4, maxres=64)
    mlp = rng.normal(0, 0.25, rc_oracle.NPARAM)
    mlp[rc_oracle.HIDDEN * 64 * 64 + 3 * 64:] = 0.0
    grid = rng.uniform(-0.5, 0.5, (rc_oracle.LEVELS, T, 2))
    rec = np.zeros((n, 16))
    rec[:, 0:3] = rng.uniform(0.5, 9.5, (n, 3))
    rec[:, 3] = rng.uniform(0.1, 1.0, n)
    d = rng.normal(size=(n, 3))
    rec[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rec[:, 8:11] = rec[:, 4:7]
    rec[:, 12:15] = rng.uniform(0, 1, (n, 3))
    return c, mlp, grid, rec


def loss_fixed_den(c, mlp, grid, rec, den):
    _, P = c.forward(mlp, grid, rec)
    p = P[:, :3]
    return np.sum((p - rec[:, 12:15]) ** 2 / den) / (3 * len(rec))


def test_oracle_gradients_match_finite_differences():
    c, mlp, grid, rec = setup()
    loss, gm, gg, P = c.loss_and_grads(mlp, grid, rec)
    den = P[:, :3] ** 2 + 0.01          # the loss treats its denominator as a constant
    rng = np.random.default_rng(1)
    h = 1e-6
    for i in list(rng.choice(rc_oracle.HIDDEN * 64 * 64, 12, replace=False)) + [rc_oracle.HIDDEN * 4096 + 5]:
        m1, m2 = mlp.copy(), mlp.copy()
        m1[i] += h
        m2[i] -= h
        fd = (loss_fixed_den(c, m1, grid, rec, den) - loss_fixed_den(c, m2, grid, rec, den)) / (2 * h)
        assert abs(fd - gm[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, gm[i])
    flat = grid.reshape(-1)
    touched = np.nonzero(gg)[0]
    for i in rng.choice(touched, 12, replace=False):
        g1, g2 = flat.copy(), flat.copy()
        g1[i] += h
        g2[i] -= h
        fd = (loss_fixed_den(c, mlp, g1.reshape(grid.shape), rec, den)
              - loss_fixed_den(c, mlp, g2.reshape(grid.shape), rec, den)) / (2 * h)
        assert abs(fd - gg[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, gg[i])


def test_levels_and_dense_indexing():
    res, dense = rc_oracle.levels(2 ** 19, 16, 2048)
    assert res[0] == 16 and res[-1] == 2048
    assert all(res[i] < res[i + 1] for i in range(15))
    assert [d > 0 for d in dense[:6]] == [True, True, True, True, True, False] or dense[4] > 0
    for r, d in zip(res, dense):
        if d:
            assert d == r + 1 and d ** 3 <= 2 ** 19


def test_sh_orthonormal_on_the_sphere():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    Y = rc_oracle.sh16(d)
    G = Y.T @ Y * (4 * np.pi / len(d))
    assert np.allclose(G, np.eye(16), atol=0.02)
