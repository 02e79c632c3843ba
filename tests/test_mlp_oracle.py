"""The FP64 restatement of the proposal network (oracle/mlp.py): its
back-propagation against central finite differences, its BF16 rounding, and
the feature layout.  The GPU training kernel is checked against it in
tests/test_proposal.py."""
import numpy as np

from oracle import mlp as M


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = M.init_params(1)
    X = rng.normal(size=(24, M.IN))
    y = (rng.uniform(size=24) < 0.3).astype(np.float64)
    _, _, g = M.forward_backward(p, X, y, pos_weight=3.0, emulate=False)
    idx = rng.choice(M.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [M.OFF["b4"][0], M.OFF["w4"][0] + 5, M.OFF["b1"][0] + 7]])
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        lp = M.forward_backward(pp, X, y, 3.0, emulate=False)[0]
        lm = M.forward_backward(pm, X, y, 3.0, emulate=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * (1 + abs(g[k])) + 1e-8, (k, fd, g[k])


def test_emulated_roundings_stay_close_to_exact():
    rng = np.random.default_rng(2)
    p = M.init_params(2)
    X = M.bf16(rng.normal(size=(256, M.IN)))
    y = (rng.uniform(size=256) < 0.4).astype(np.float64)
    l0, z0, g0 = M.forward_backward(p, X, y, 8.0, emulate=False)
    l1, z1, g1 = M.forward_backward(p, X, y, 8.0, emulate=True)
    assert abs(l1 - l0) <= 2e-2 * abs(l0)
    cos = g0 @ g1 / np.linalg.norm(g0) / np.linalg.norm(g1)
    assert cos > 0.999


def test_bf16_round_to_nearest_even():
    one = 1.0
    assert M.bf16(one) == 1.0
    assert M.bf16(1.0 + 2.0 ** -8) == 1.0            # tie -> even
    assert M.bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6  # tie -> even (up)
    assert M.bf16(1.0 + 2.0 ** -8 + 2.0 ** -20) == 1.0 + 2.0 ** -7
    assert M.bf16(-2.5) == -2.5
    b = M.bf16_bits(np.array([1.0, -2.0, 0.5]))
    assert list(b) == [0x3F80, 0xC000, 0x3F00]
    assert list(M.from_bf16_bits(b)) == [1.0, -2.0, 0.5]


def test_feature_layout():
    a = np.array([[0.1, -0.2, 0.3]])
    b = np.array([[0.4, 0.2, -0.1]])
    X = M.segment_features(a, b)
    assert X.shape == (1, 64)
    assert X[0, 0] == 0.1 and np.isclose(X[0, 1], np.sin(np.pi * 0.1))
    assert np.isclose(X[0, 8], np.cos(np.pi * 0.1 * 8))
    d = (b - a) / np.linalg.norm(b - a)
    assert np.allclose(X[0, 54:57], d[0]) and X[0, 57] == 1.0
    assert np.all(X[0, 58:] == 0)
