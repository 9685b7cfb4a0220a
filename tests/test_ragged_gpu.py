"""Ragged batches: pairs of arbitrary sizes through the persistent,
graph-captured plan and through per-pair launches, against the oracle."""
import os

import numpy as np
import pytest

from helpers import rel_to_max
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import xcorr  # noqa: E402


def ragged_batch(n_pairs, lo, hi, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    lefts, rights = [], []
    for _ in range(n_pairs):
        hl, wl, hr, wr = rng.integers(lo, hi + 1, size=4)
        lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(dtype))
        rights.append(rng.uniform(-1, 1, (hr, wr)).astype(dtype))
    # edge shapes: strips and single elements
    lefts += [np.ones((1, 37), dtype), rng.uniform(-1, 1, (45, 1)).astype(dtype), np.full((1, 1), 2, dtype)]
    rights += [rng.uniform(-1, 1, (3, 5)).astype(dtype), rng.uniform(-1, 1, (1, 1)).astype(dtype),
               rng.uniform(-1, 1, (17, 9)).astype(dtype)]
    return lefts, rights, [(i, i) for i in range(len(lefts))]


@pytest.fixture(autouse=True)
def isolated_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("XC_AUTOTUNE_CACHE", str(tmp_path / "autotune.jsonl"))


def check_outputs(outs, lefts, rights, pairs, dtype="f32acc64", tol=1e-5):
    refs = oracle.run_pairs([lefts[a] for a, _ in pairs], [rights[b] for _, b in pairs], dtype=dtype, threads=8)
    assert len(outs) == len(refs)
    for k, (o, r) in enumerate(zip(outs, refs)):
        assert o.shape == r.shape, k
        assert rel_to_max(o, r) <= tol, k


def test_ragged_plan_matches_oracle_and_per_pair_launches():
    lefts, rights, pairs = ragged_batch(24, 5, 90, 7)
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    plan.execute()
    torch.cuda.synchronize()
    outs = plan.outputs()
    check_outputs(outs, lefts, rights, pairs)
    base = torch.zeros_like(plan.out)
    plan.per_pair(base)
    torch.cuda.synchronize()
    check_outputs(plan.outputs(base), lefts, rights, pairs)
    plan.close()


def test_ragged_autotune_and_graph_replay_with_new_data():
    lefts, rights, pairs = ragged_batch(16, 10, 140, 8)
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    shape, ms = plan.autotune()
    assert 0 <= shape < plan.describe()["n_variants"] and ms > 0
    assert plan.describe()["index"] == shape
    # the graph re-reads the bound input buffers on every execution
    rng = np.random.default_rng(9)
    lefts2 = [rng.uniform(-1, 1, a.shape).astype(np.float32) for a in lefts]
    plan.left.copy_(torch.from_numpy(xcorr.pack(lefts2)[0]))
    for _ in range(2):
        plan.execute()
    torch.cuda.synchronize()
    check_outputs(plan.outputs(), lefts2, rights, pairs)
    # a second plan of the same batch takes the cached decision
    plan2 = xcorr.RaggedPlan(lefts, rights, pairs)
    shape2, ms2 = plan2.autotune()
    assert shape2 == shape and ms2 < 0
    assert os.path.exists(os.environ["XC_AUTOTUNE_CACHE"])
    plan.close()
    plan2.close()


def test_ragged_fp64():
    lefts, rights, pairs = ragged_batch(8, 4, 40, 10, np.float64)
    plan = xcorr.RaggedPlan(lefts, rights, pairs, dtype="f64")
    plan.execute()
    torch.cuda.synchronize()
    check_outputs(plan.outputs(), lefts, rights, pairs, dtype="f64", tol=1e-12)
    plan.close()


def test_ragged_shared_matrices_n_to_m_style():
    """Pairs may reuse matrices (a ragged n_to_m: every left with every right)."""
    rng = np.random.default_rng(11)
    lefts = [rng.uniform(-1, 1, (h, w)).astype(np.float32) for h, w in [(20, 33), (7, 64), (50, 12)]]
    rights = [rng.uniform(-1, 1, (h, w)).astype(np.float32) for h, w in [(9, 9), (31, 17)]]
    pairs = [(a, b) for a in range(3) for b in range(2)]
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    plan.execute()
    torch.cuda.synchronize()
    check_outputs(plan.outputs(), lefts, rights, pairs)
    plan.close()


def test_ragged_largest_pairs_match_oracle():
    """Pairs with every side near the top of the U{16..512} range of the
    512-pair batch, where FP32 chains are longest (the batch's checks in the
    bench cover its 8 largest pairs the same way)."""
    rng = np.random.default_rng(44)
    lefts = [rng.uniform(-1, 1, (512, 497)).astype(np.float32), rng.uniform(-1, 1, (479, 512)).astype(np.float32)]
    rights = [rng.uniform(-1, 1, (505, 488)).astype(np.float32), rng.uniform(-1, 1, (512, 509)).astype(np.float32)]
    pairs = [(0, 0), (1, 1)]
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    plan.execute()
    base = torch.zeros_like(plan.out)
    plan.per_pair(base)
    torch.cuda.synchronize()
    # one pair at a time, its rows over all host threads
    refs = [oracle.run_mode("one_to_one", a, b, threads=os.cpu_count() or 1)[0] for a, b in zip(lefts, rights)]
    for got, got_pp, ref in zip(plan.outputs(), plan.outputs(base), refs):
        assert rel_to_max(got, ref) <= 1e-5
        assert rel_to_max(got_pp, ref) <= 1e-5
    plan.close()


def test_ragged_split_routes_match_oracle():
    """FP32 plans can route the pairs with the most multiply-adds through the
    split-BF16 path (one_to_one calls on side streams, captured into the same
    graph as the plain kernel's launch for the other pairs).  Every route, with
    either tile shape, matches the oracle on every pair; the outputs start as
    NaN, so a pair that no branch writes fails."""
    rng = np.random.default_rng(12)
    sides = [(160, 150, 170, 140),   # 5.7e8 multiply-adds: routes 3 and 4
             (300, 280, 260, 290),   # 6.3e9: every route
             (64, 70, 80, 90),       # 3.2e7: plain kernel only
             (12, 30, 7, 9),
             (200, 60, 180, 70),     # 1.5e8: route 4
             (1, 300, 1, 290),
             (4, 3000, 4, 2000),     # 9.6e7, a wide strip: route 4
             (130, 128, 127, 129)]   # 2.73e8: routes 3 and 4
    lefts = [rng.uniform(-1, 1, (a, b)).astype(np.float32) for a, b, _, _ in sides]
    rights = [rng.uniform(-1, 1, (c, d)).astype(np.float32) for _, _, c, d in sides]
    pairs = [(i, i) for i in range(len(sides))]
    refs = oracle.run_pairs(lefts, rights, threads=os.cpu_count() or 1)
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    n = plan.describe()["n_variants"]
    assert n == 10  # 2 tile shapes x 5 routes
    routed = []
    for v in range(n):
        d = plan.describe(v)
        assert d["index"] == v and d["tile_shape"] == v % 2
        routed.append(d["tc_pairs"])
        plan.select(v)
        plan.out.fill_(float("nan"))
        plan.execute()
        torch.cuda.synchronize()
        for k, (got, ref) in enumerate(zip(plan.outputs(), refs)):
            assert got.shape == ref.shape
            assert rel_to_max(got, ref) <= 1e-5, (v, k)
    assert routed == [0, 0, 1, 1, 1, 1, 3, 3, 5, 5]
    plan.close()


def test_ragged_fp64_plans_keep_every_pair_on_the_plain_kernel():
    lefts, rights, pairs = ragged_batch(3, 100, 140, 13, np.float64)
    plan = xcorr.RaggedPlan(lefts, rights, pairs, dtype="f64")
    assert plan.describe()["n_variants"] == 1
    with pytest.raises(xcorr.XcError):
        plan.select(1)
    plan.close()


_SWITCH_SCRIPT = """
import json, sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + '/cross-corr_gb300']
import numpy as np, torch, xcorr
from oracle import oracle
rng = np.random.default_rng(14)
shapes = [(150, 140, 130, 160), (120, 110, 100, 130), (30, 40, 20, 10)]
lefts = [rng.uniform(-1, 1, (a, b)).astype(np.float32) for a, b, _, _ in shapes]
rights = [rng.uniform(-1, 1, (c, d)).astype(np.float32) for _, _, c, d in shapes]
plan = xcorr.RaggedPlan(lefts, rights, [(i, i) for i in range(3)])
n = plan.describe()["n_variants"]
err = None
if n > 2:
    plan.select(n - 2)  # tile shape 0, the pairs of at least 2^26 multiply-adds on the split path
    plan.out.fill_(float("nan"))
    plan.execute()
    torch.cuda.synchronize()
    refs = oracle.run_pairs(lefts, rights, threads=8)
    err = max(float(np.nanmax(np.abs(o - r)) / np.abs(r).max()) if not np.isnan(o).any() else 1.0
              for o, r in zip(plan.outputs(), refs))
print(json.dumps({"n_variants": n, "tc_pairs": plan.describe(n - 2 if n > 2 else 0)["tc_pairs"], "err": err}))
plan.close()
"""


@pytest.mark.parametrize("env,variants", [({"XC_RAGGED_TC": "0"}, 2), ({"XC_RAGGED_TC_STREAMS": "1"}, 10)])
def test_ragged_environment_switches(env, variants):
    """XC_RAGGED_TC=0 leaves FP32 plans with the plain kernel only (the two
    tile shapes); XC_RAGGED_TC_STREAMS=1 puts every routed call on one side
    stream, with the same results.  The switches are read once per process,
    so each case runs in a child process."""
    import json
    import subprocess
    import sys

    from conftest import ROOT

    out = subprocess.run([sys.executable, "-c", _SWITCH_SCRIPT, ROOT], env={**os.environ, **env}, cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["n_variants"] == variants
    if variants > 2:
        assert res["tc_pairs"] == 2
        assert res["err"] <= 1e-5
    else:
        assert res["tc_pairs"] == 0
