"""The method selector on the GPU: the MLP kernels against the numpy oracle,
training from scratch on the committed GB300 timing dataset, and what the
trained network gains over selection without it."""
import os

import numpy as np
import pytest

from oracle import mlp_oracle

import xcorr
from xcorr import selector

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DATASET = os.path.join(os.path.dirname(HERE), "cross-corr_gb300", "selector", "data", "gb300_timings.npz")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def _case(seed, n=53):
    rng = np.random.default_rng(seed)
    p = mlp_oracle.init(seed).astype(np.float32)
    x = rng.uniform(0, 1, (n, 8)).astype(np.float32)
    t = rng.standard_normal((n, mlp_oracle.OUT)).astype(np.float32)
    m = (rng.random((n, mlp_oracle.OUT)) > 0.25).astype(np.float32)
    return p, x, t, m


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_forward_matches_oracle(seed):
    p, x, _, _ = _case(seed)
    y = selector.predict(p, x)
    ref = mlp_oracle.forward(p.astype(np.float64), x.astype(np.float64))[0]
    assert np.max(np.abs(y - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gradient_matches_oracle(seed):
    p, x, t, m = _case(seed)
    tr = selector.Trainer(p)
    g, loss = tr.gradient(_dev(x), _dev(t), _dev(m))
    torch.cuda.synchronize()
    ref_loss, ref_g = mlp_oracle.loss_and_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64),
                                               m.astype(np.float64))
    g = g.cpu().numpy().astype(np.float64)
    # FP32 products summed by atomics in arbitrary order: a relative bound on the largest entry
    assert np.max(np.abs(g - ref_g)) <= 2e-5 * np.max(np.abs(ref_g))
    assert abs(float(loss.item()) - ref_loss) <= 1e-5 * abs(ref_loss)


def test_gradient_all_masked_is_zero():
    p, x, t, _ = _case(3)
    tr = selector.Trainer(p)
    g, loss = tr.gradient(_dev(x), _dev(t), _dev(np.zeros((x.shape[0], mlp_oracle.OUT))))
    assert float(g.abs().max().item()) == 0.0 and float(loss.item()) == 0.0


def test_adam_step_matches_formula():
    p, x, t, m = _case(4)
    tr = selector.Trainer(p)
    X, T, M = _dev(x), _dev(t), _dev(m)
    ref_p = p.astype(np.float64)
    mo = np.zeros_like(ref_p)
    v = np.zeros_like(ref_p)
    lr = 1e-3
    for step in range(1, 4):
        # the oracle's Adam sees the gradient the GPU computes at the GPU's current parameters
        g, _ = tr.gradient(X, T, M)
        gh = g.cpu().numpy().astype(np.float64)
        mo = 0.9 * mo + 0.1 * gh
        v = 0.999 * v + 0.001 * gh * gh
        ref_p = tr.p.cpu().numpy().astype(np.float64) - lr * (mo / (1 - 0.9 ** step)) / (
            np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
        tr.t = step
        xcorr.check(xcorr.lib().xc_mlp_adam_step(tr.p.data_ptr(), tr.g.data_ptr(), tr.m.data_ptr(), tr.v.data_ptr(),
                                                 step, lr, torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        assert np.max(np.abs(tr.p.cpu().numpy() - ref_p)) <= 1e-6


def test_training_reduces_loss_like_oracle_descent():
    """A few full-batch steps on the GPU decrease the oracle's loss."""
    p, x, t, m = _case(5, n=200)
    tr = selector.Trainer(p)
    before = mlp_oracle.loss_and_grad(p.astype(np.float64), x, t, m)[0]
    tr.fit(x, t, m, steps=200, lr=3e-3)
    after = mlp_oracle.loss_and_grad(tr.params().astype(np.float64), x, t, m)[0]
    assert after < 0.5 * before


@pytest.fixture(scope="module")
def trained():
    """Train from scratch on the committed dataset (held-out split untouched)."""
    if not os.path.exists(DATASET):
        pytest.skip("timing dataset not collected")
    X, T, M, times = selector.load_dataset(DATASET)
    tr_idx, te_idx = selector.split(len(X), 0)
    Ts, _, _ = selector.standardise(T[tr_idx], M[tr_idx])
    trainer = selector.Trainer(selector.init_params(0))
    trainer.fit(X[tr_idx], Ts, M[tr_idx], steps=3000)
    return trainer.params(), X, M, times, te_idx


def test_trained_selector_within_10_percent_of_exhaustive_autotune(trained):
    params, X, M, times, te = trained
    chosen = selector.choose(selector.predict(params, X[te]), M[te])
    total, mean = selector.regret(times[te], chosen)
    assert total <= 0.10, total
    assert mean <= 0.10, mean


def test_trained_selector_beats_selection_without_it(trained):
    """What the network gains on the held-out workloads.  Without it, a new
    problem either runs a fixed choice or pays for the exhaustive autotune
    (XC_METHOD_AUTO's first call for a problem when no network is installed),
    which runs every supported candidate once before the best one.  The
    network's picks must cost far less than the autotune, and less than the
    best fixed candidate."""
    params, X, M, times, te = trained
    chosen = selector.choose(selector.predict(params, X[te]), M[te])
    t = times[te]
    ours = t[np.arange(len(te)), chosen].sum()
    best = t.min(axis=1).sum()
    autotune_cost = (np.where(M[te] > 0, t, 0).sum(axis=1) + t.min(axis=1)).sum()
    fft = selector.ALGO_NAMES.index("fft")
    fixed = min(t[np.arange(len(te)), np.where(M[te][:, k] > 0, k, fft)].sum() for k in range(selector.N_OUT))
    assert ours <= 1.10 * best
    assert ours < 0.5 * autotune_cost
    assert ours < fixed


def test_live_selection_matches_exhaustive_autotune(trained):
    """Live on this GPU: for held-out workloads of moderate size, the method
    the network picks runs within 10% (in total) of the method the exhaustive
    autotune finds fastest."""
    params, X, M, times, te = trained
    z = np.load(DATASET)
    picked = [j for j in te if times[j, 0] < 0.05 and 2e-4 < times[j].min() < 0.02][:8]
    assert len(picked) >= 4
    selector.install(params)
    total_auto, total_best = 0.0, 0.0
    try:
        for j in picked:
            mode = str(z["modes"][j])
            sl, sr, b = int(z["sides_left"][j]), int(z["sides_right"][j]), int(z["batch"][j])
            n_l, n_r = selector.counts(mode, b)
            rng = np.random.default_rng(int(j))
            left = torch.from_numpy(rng.random((n_l, sl, sl), dtype=np.float32)).cuda()
            right = torch.from_numpy(rng.random((n_r, sr, sr), dtype=np.float32)).cuda()
            out = xcorr.correlate(mode, left, right, method="auto")
            best, best_ms = selector.autotune(mode, left, right, out)
            m = selector.select(mode, "f32", (sl, sl), n_l, (sr, sr), n_r)
            auto_ms = selector.time_algo(mode, left, right, out, m)
            best_ms = selector.time_algo(mode, left, right, out, best)
            total_auto += auto_ms
            total_best += best_ms
    finally:
        selector.install("builtin")
    assert total_auto <= 1.10 * total_best, (total_auto, total_best)


def test_auto_dispatch_uses_loaded_weights(trained):
    params, X, M, times, te = trained
    pred = selector.predict(params, X[te])
    want = selector.choose(pred, M[te])
    z = np.load(DATASET)
    selector.install(params)
    try:
        for j, w in zip(te[:64], want[:64]):
            mode = str(z["modes"][j])
            sl, sr, b = int(z["sides_left"][j]), int(z["sides_right"][j]), int(z["batch"][j])
            n_l, n_r = selector.counts(mode, b)
            got = selector.select(mode, "f32", (sl, sl), n_l, (sr, sr), n_r)
            # the C++ forward and the GPU forward agree up to rounding; skip near-ties
            gap = np.sort(np.where(M[j] > 0, pred[list(te).index(j)], np.inf))[:2]
            if gap[1] - gap[0] > 1e-3:
                assert got == selector.ALGO_NAMES[w]
    finally:
        selector.install(None)
    try:
        # no network and no tuning record: undecided, the first call autotunes
        assert selector.select("one_to_one", "f32", (64, 64), 1, (640, 640), 1) == "auto"
        rng = np.random.default_rng(11)
        left = torch.from_numpy(rng.random((1, 64, 64), dtype=np.float32)).cuda()
        right = torch.from_numpy(rng.random((1, 40, 40), dtype=np.float32)).cuda()
        out = xcorr.correlate("one_to_one", left, right, method="auto")
        torch.cuda.synchronize()
        picked = selector.select("one_to_one", "f32", (64, 64), 1, (40, 40), 1)
        assert picked in selector.ALGO_NAMES
        ref = xcorr.correlate("one_to_one", left, right, method="fft")
        assert float((out - ref).abs().max()) <= 1e-5 * float(ref.abs().max())
    finally:
        selector.install("builtin")
