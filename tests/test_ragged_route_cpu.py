"""The split-BF16 routes of a ragged plan, on the CPU.

An FP32 ragged plan can send its pairs with the most multiply-adds to the
split tensor-core path, as per-pair calls on side streams captured into the
plan's graph (`csrc/ragged_route.h`, the header `ragged.cu` plans them with).
This compiles `ragged_route_check.cpp` against that header with the host C++
compiler and checks: route r takes exactly the pairs the split path accepts
with at least 2^(34-2r) multiply-adds; every routed pair goes to one stream
once; each stream issues its pairs longest first; and the least-loaded deal
keeps the streams within one call's cost of each other.  No GPU needed."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "cross-corr_gb300", "csrc")
FIXED = 2.0 ** 26  # the fixed cost of one call, in multiply-adds


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("route") / "ragged_route_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I" + CSRC, os.path.join(HERE, "ragged_route_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def plan(exe, route, n_streams, macs, oks):
    line = f"{route} {n_streams} {len(macs)} " + " ".join(f"{m:.0f} {int(o)}" for m, o in zip(macs, oks))
    out = subprocess.run([exe], input=line + "\n", capture_output=True, text=True, check=True).stdout.split()
    threshold, n = float(out[0]), int(out[1])
    streams, cur = [], None
    for tok in out[2:]:
        if tok == "|":
            cur = []
            streams.append(cur)
        else:
            cur.append(int(tok))
    assert len(streams) == n
    return threshold, streams


def batch_512():
    """Multiply-adds of the bench's 512-pair batch (every side from U{16..512}, seed 4)."""
    rng = np.random.default_rng(4)
    macs = []
    for _ in range(512):
        hl, wl, hr, wr = rng.integers(16, 513, size=4)
        rng.uniform(-1, 1, (hl, wl))
        rng.uniform(-1, 1, (hr, wr))
        macs.append(float(hl) * wl * hr * wr)
    return macs


@pytest.mark.parametrize("route", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("n_streams", [1, 4, 8])
def test_routes_take_the_right_pairs_and_deal_them_evenly(checker, route, n_streams):
    macs = batch_512()
    oks = [(i % 17) != 3 for i in range(len(macs))]  # some pairs the split path would refuse
    threshold, streams = plan(checker, route, n_streams, macs, oks)
    assert threshold == (0.0 if route == 0 else 2.0 ** (34 - 2 * route))
    want = {i for i, (m, o) in enumerate(zip(macs, oks)) if route > 0 and o and m >= threshold}
    got = [i for s in streams for i in s]
    assert len(got) == len(set(got)) and set(got) == want
    for s in streams:
        assert all(macs[a] >= macs[b] for a, b in zip(s, s[1:])), "a stream issues its pairs longest first"
    if want:
        loads = [sum(macs[i] + FIXED for i in s) for s in streams]
        assert max(loads) - min(loads) <= max(macs[i] for i in want) + FIXED


def test_the_autotuned_route_of_the_512_pair_batch(checker):
    """The route the autotuner picks on the GB300 (2^28) sends 448 of the 512
    pairs, with 99.7% of the multiply-adds, to the split path."""
    macs = batch_512()
    _, streams = plan(checker, 3, 8, macs, [True] * len(macs))
    routed = [i for s in streams for i in s]
    assert len(routed) == 448
    assert sum(macs[i] for i in routed) / sum(macs) > 0.996
    assert all(len(s) > 0 for s in streams)


def test_ties_keep_pair_order(checker):
    _, (s,) = plan(checker, 4, 1, [2.0 ** 27] * 5, [True] * 5)
    assert s == [0, 1, 2, 3, 4]
