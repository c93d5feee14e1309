"""The MLP oracle's analytic backward pass against central finite differences (FP64, no
rounding): the oracle is trusted only after this."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = M.init_params(1).astype(np.float64)
    p[M.OFF_W4:M.OFF_B4] *= 3.0  # larger output layer so every gradient block is well above noise
    x = rng.uniform(-1, 1, (32, M.IN))
    t = rng.normal(0, 0.5, (32, 3))
    g = M.gradients(p, x, t, bf16=False)
    idx = np.concatenate([rng.choice(np.arange(o, o + 64), 6, replace=False)
                          for o in (M.OFF_W1, M.OFF_B1, M.OFF_W2, M.OFF_B2, M.OFF_W3, M.OFF_B3)]
                         + [np.arange(M.OFF_W4, M.OFF_W4 + 6), np.arange(M.OFF_B4, M.OFF_B4 + 3)])
    for i in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss(pp, x, t) - M.loss(pm, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_padding_gradients_are_zero():
    rng = np.random.default_rng(1)
    p = M.init_params(2).astype(np.float64)
    x = rng.uniform(-1, 1, (16, M.IN))
    t = rng.normal(0, 0.5, (16, 3))
    g = M.gradients(p, x, t, bf16=False)
    W1 = g[M.OFF_W1:M.OFF_B1].reshape(M.H, M.K0)
    assert np.all(W1[:, M.IN:] == 0)
    W4 = g[M.OFF_W4:M.OFF_B4].reshape(M.NO, M.H)
    assert np.all(W4[3:] == 0) and np.all(g[M.OFF_B4 + 3:] == 0)
