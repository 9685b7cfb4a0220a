"""Selector pieces that need no GPU: the numpy oracle's gradient against
finite differences and the feature function of the C ABI."""
import ctypes

import numpy as np

from oracle import mlp_oracle

import xcorr


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = mlp_oracle.init(1).astype(np.float64)
    x = rng.uniform(0, 1, (6, 8))
    t = rng.standard_normal((6, 3))
    m = (rng.random((6, 3)) > 0.2).astype(np.float64)
    loss, g = mlp_oracle.loss_and_grad(p, x, t, m)
    idx = rng.choice(p.size, 40, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = mlp_oracle.loss_and_grad(q, x, t, m)
        q[i] -= 2 * eps
        lm, _ = mlp_oracle.loss_and_grad(q, x, t, m)
        assert abs((lp - lm) / (2 * eps) - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_parameter_count_matches_header():
    assert mlp_oracle.N_PARAMS == 64 * 8 + 64 + 64 * 64 + 64 + 3 * 64 + 3


def test_selector_features():
    f = (ctypes.c_float * 8)()
    xcorr.check(xcorr.lib().xc_selector_features(xcorr.MODES["n_to_m"], xcorr.size2(256, 256), 2,
                                                 xcorr.size2(64, 128), 8, f))
    v = np.array(f[:])
    assert np.allclose(v[:3], [16 / 22, 13 / 22, 4 / 8])
    assert list(v[3:7]) == [0, 0, 0, 1]
    assert np.isclose(v[7], (16 + 13 + 4) / 64)
    assert xcorr.lib().xc_selector_features(xcorr.MODES["n_to_mn"], xcorr.size2(4, 4), 3, xcorr.size2(4, 4), 4,
                                            f) == 1
