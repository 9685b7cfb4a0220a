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
    t = rng.standard_normal((6, mlp_oracle.OUT))
    m = (rng.random((6, mlp_oracle.OUT)) > 0.2).astype(np.float64)
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
    assert mlp_oracle.N_PARAMS == 64 * 8 + 64 + 64 * 64 + 64 + 7 * 64 + 7


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


def test_candidate_table_matches_binding():
    """xc_algorithm's candidates are the network's outputs, in the order the
    Python side names them."""
    from xcorr import selector

    assert selector.N_OUT == mlp_oracle.OUT
    for k, name in enumerate(selector.ALGO_NAMES):
        a = xcorr.Algo()
        xcorr.check(xcorr.lib().xc_algorithm(k, ctypes.byref(a)))
        want = selector.algo_struct(name)
        assert (a.method, a.tile) == (want.method, want.tile), name
    assert xcorr.lib().xc_algorithm(len(selector.ALGO_NAMES), ctypes.byref(xcorr.Algo())) == 1


def test_correlate_algo_rejects_invalid_tiles_before_any_launch():
    """Tile checks run on the host: no GPU is touched (the pointers are never
    dereferenced)."""
    dummy = ctypes.c_void_p(256)
    s = xcorr.size2(16, 16)
    for method, tile in (("direct", 4), ("direct", -1), ("fft", 1), ("tc_bf16x3", 3), ("tc_tf32x3", 2048)):
        a = xcorr.Algo(xcorr.METHODS[method], tile)
        st = xcorr.lib().xc_correlate_algo(xcorr.MODES["one_to_one"], xcorr.DTYPES["f32"], a, dummy, s, 1, dummy, s,
                                           1, dummy, None, 0, None)
        assert st == 1, (method, tile)
        assert "tile" in xcorr.lib().xc_last_error().decode()


def test_timing_dataset_names_the_candidates():
    """The committed GB300 timing dataset has one column per candidate, in
    the network's output order, and every workload has a finite time for the
    FFT path (which supports every problem)."""
    import os

    from xcorr import selector

    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cross-corr_gb300", "selector",
                        "data", "gb300_timings.npz")
    z = np.load(path)
    assert [str(a) for a in z["algorithms"]] == selector.ALGO_NAMES
    n = len(z["modes"])
    assert int(z["n_done"]) == n == 4097
    t = z["times"]
    assert t.shape == (n, selector.N_OUT)
    assert np.isfinite(t[:, selector.ALGO_NAMES.index("fft")]).all()
    assert (t > 0).all()
