"""CPU checks of the network oracle itself: BF16 rounding, the gradient formulas against
finite differences, and the Adam update."""

import numpy as np

from oracle import surrogate as S


def test_bf16_rounding_ties_to_even():
    one = np.float32(1.0)
    ulp = np.float32(2.0 ** -7)
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -8 + 2.0 ** -20], np.float32)
    r = S.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie -> even mantissa
    assert r[2] == float(one + 2 * ulp)      # tie with odd lower neighbour -> up
    assert r[3] == -2.5
    assert r[4] == float(one + ulp)          # above the tie -> up


def _small_grid():
    res = [4 + 3 * l for l in range(S.LEVELS)]
    T = 1 << 10
    dense = sum(1 << l for l, r in enumerate(res) if (r + 1) ** 3 <= T)
    return S.Grid(res, dense, T, clamp=0.5)


def test_dense_and_hashed_indices():
    g = _small_grid()
    u = g.unit(np.array([[-2.0, -2.0, -2.0], [2.0, 2.0, 2.0], [0.0, 0.0, 0.0]]))
    idx, w = g.corners(u, 0)                 # level 0 is dense: 5^3 corners
    assert idx[0, 0] == 0 and idx[1, 7] == 5 ** 3 - 1
    np.testing.assert_allclose(w.sum(1), 1.0, atol=1e-6)
    idx, _ = g.corners(u, S.LEVELS - 1)      # hashed
    assert idx.max() < g.T


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    g = _small_grid()
    table = rng.uniform(-1, 1, S.LEVELS * g.T * 2)
    mlp = np.zeros(S.PARAMS)
    for off, out, inp in ((S.W1, 64, 32), (S.W2, 64, 64), (S.W3, 64, 64), (S.W4, 1, 64)):
        a = np.sqrt(6.0 / (inp + out))
        mlp[off:off + out * inp] = rng.uniform(-a, a, out * inp)
    mlp[S.B1:S.W2] = rng.uniform(-0.1, 0.1, 64)
    mlp[S.B4] = 0.05
    smp = np.concatenate([rng.uniform(-1.8, 1.8, (48, 3)), rng.uniform(-0.6, 0.6, (48, 1))], 1)
    gt, gm, _ = S.gradients(g, table, mlp, smp, rounded=False)

    def loss(t, m):
        a = S.forward(g, t, m, smp[:, :3], rounded=False)
        tgt = np.clip(smp[:, 3].astype(np.float32).astype(np.float64), -0.5, 0.5)
        return np.mean((a["s"] - tgt) ** 2)

    h = 1e-6
    for k in rng.choice(S.PARAMS, 40, replace=False):
        mp, mm = mlp.copy(), mlp.copy()
        mp[k] += h
        mm[k] -= h
        fd = (loss(table, mp) - loss(table, mm)) / (2 * h)
        assert abs(fd - gm[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gm[k])
    live = np.flatnonzero(np.abs(gt) > 1e-4)
    for k in rng.choice(live, 40, replace=False):
        tp, tm = table.copy(), table.copy()
        tp[k] += h
        tm[k] -= h
        fd = (loss(tp, mlp) - loss(tm, mlp)) / (2 * h)
        assert abs(fd - gt[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gt[k])


def test_adam_first_step_is_signed_rate():
    g = np.array([0.5, -1e-3, 0.0, 2.0])
    p, m, v = S.adam(np.ones(4), g, np.zeros(4), np.zeros(4), 1, 0.01)
    np.testing.assert_allclose(p, [0.99, 1.01, 1.0, 0.99], rtol=0, atol=1e-12)
    np.testing.assert_allclose(m, 0.1 * g)
    np.testing.assert_allclose(v, 0.01 * g * g)
