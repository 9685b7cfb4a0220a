"""xc_correlate_host_async / xc_host_wait: host-buffer problems as a stream,
two calls in flight per thread (one call's copies under the other's kernel).
Every result must equal what the synchronous host-buffer call gives, within
the tolerances the other host-buffer tests use, and the oracle's within 1e-5."""
import ctypes

import numpy as np
import pytest

from helpers import rel_to_max, seeded
from oracle import oracle

import xcorr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def pinned(a):
    """A pinned copy of `a` and the tensor that owns its memory."""
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t.numpy(), t


def out_shape(mode, left, right):
    return (xcorr.output_count(mode, left.shape[0], right.shape[0]), left.shape[1] + right.shape[1] - 1,
            left.shape[2] + right.shape[2] - 1)


# (mode, method, n_left, n_right, left side, right shape, seed): the split
# cases of 16 MiB of output or more copy their output out in bands
PROBLEMS = [
    ("one_to_many", "tc_bf16x3", 1, 20, 256, (256, 256), 61),
    ("n_to_m", "direct", 3, 4, 48, (40, 56), 62),
    ("one_to_many", "fft", 1, 6, 100, (90, 100), 63),
    ("one_to_many", "tc_bf16x3", 1, 18, 240, (256, 250), 64),
    ("n_to_mn", "tc_tf32x3", 2, 16, 200, (210, 220), 65),
    ("one_to_one", "auto", 1, 1, 70, (70, 70), 66),
    ("n_to_m", "direct", 2, 3, 40, (36, 44), 67, np.float64),
    ("n_to_mn", "fft", 2, 4, 64, (64, 64), 68, np.float64),
]


def make(problem):
    mode, method, n_l, n_r, side, rshape, seed = problem[:7]
    dtype = problem[7] if len(problem) > 7 else np.float32
    left = seeded((n_l, side, side), seed, dtype=dtype)
    right = seeded((n_r,) + rshape, seed + 100, dtype=dtype)
    return mode, method, left, right


def test_stream_of_problems_matches_the_synchronous_call():
    keep = []
    calls = []
    for p in PROBLEMS:
        mode, method, left, right = make(p)
        hl, tl = pinned(left)
        hr, tr = pinned(right)
        ho, to = pinned(np.full(out_shape(mode, left, right), np.nan, left.dtype))
        keep += [tl, tr, to]
        calls.append((mode, method, left, right, ho, xcorr.correlate_host_async(mode, hl, hr, ho, method=method)))
    # wait newest first: the older calls were completed by the later ones
    for mode, method, left, right, ho, t in reversed(calls):
        xcorr.host_wait(t)
    for mode, method, left, right, ho, t in calls:
        assert np.isfinite(ho).all(), (mode, method)
        ref = xcorr.correlate_host(mode, left, right, method=method)
        assert rel_to_max(ho, ref) <= 4e-6, (mode, method)
        k = min(2, ho.shape[0])  # the oracle on the first outputs
        pairs = [oracle.pair_of_output(mode, left.shape[0], right.shape[0], o) for o in range(k)]
        f64 = left.dtype == np.float64
        exact = oracle.run_pairs([left[a] for a, _ in pairs], [right[b] for _, b in pairs],
                                 dtype="f64" if f64 else "f32acc64", threads=8)
        for o in range(k):
            # FP64 bounds of the parity tests: 1e-12 (plain kernel), 1e-10 (FFT)
            tol = (1e-10 if method == "fft" else 1e-12) if f64 else 1e-5
            assert rel_to_max(ho[o], exact[o]) <= tol, (mode, method, o)


def test_pipeline_reuses_each_slot_for_the_same_problem():
    """Ten calls of one banded problem, alternating two output buffers and
    two input sets, waited in order: every output equals its input set's."""
    mode, method, left, right = make(PROBLEMS[0])
    left2, right2 = left[:, ::-1].copy(), right[::-1].copy()
    ins = [tuple(pinned(a) for a in (left, right)), tuple(pinned(a) for a in (left2, right2))]
    outs = [pinned(np.empty(out_shape(mode, left, right), np.float32)) for _ in range(2)]
    refs = [xcorr.correlate_host(mode, left, right, method=method),
            xcorr.correlate_host(mode, left2, right2, method=method)]
    pending = []
    for i in range(10):
        (hl, _), (hr, _) = ins[i % 2]
        ho = outs[i % 2][0]
        if len(pending) == 2:  # the buffer about to be reused: its result first
            j, t = pending.pop(0)
            xcorr.host_wait(t)
            assert rel_to_max(outs[j % 2][0], refs[j % 2]) <= 4e-6, j
        pending.append((i, xcorr.correlate_host_async(mode, hl, hr, ho, method=method)))
    for j, t in pending:
        xcorr.host_wait(t)
        assert rel_to_max(outs[j % 2][0], refs[j % 2]) <= 4e-6, j


def test_tickets():
    L = xcorr.lib()
    mode, method, left, right = make(PROBLEMS[1])
    hl, _tl = pinned(left)
    hr, _tr = pinned(right)
    ho, _to = pinned(np.empty(out_shape(mode, left, right), np.float32))
    t = xcorr.correlate_host_async(mode, hl, hr, ho, method=method)
    xcorr.host_wait(t)
    xcorr.host_wait(t)  # waiting again is fine
    assert L.xc_host_wait(ctypes.c_uint64(0)) == 1
    assert L.xc_host_wait(ctypes.c_uint64(t + 1000)) == 1
    assert L.xc_correlate_host_async(xcorr.MODES[mode], 0, xcorr.METHODS[method], hl.ctypes.data,
                                     xcorr.size2(48, 48), 3, hr.ctypes.data, xcorr.size2(40, 56), 4,
                                     ho.ctypes.data, None, None) == 1  # NULL ticket


def test_chunked_problem_completes_inside_the_call(monkeypatch):
    """Problems cut into chunks run to completion before the async call
    returns; the ticket is then already complete."""
    monkeypatch.setenv("XC_HOST_CHUNKS", "2")
    mode, method, left, right = make(PROBLEMS[2])
    hl, _tl = pinned(left)
    hr, _tr = pinned(right)
    ho, _to = pinned(np.full(out_shape(mode, left, right), np.nan, np.float32))
    t = xcorr.correlate_host_async(mode, hl, hr, ho, method=method)
    assert np.isfinite(ho).all()
    xcorr.host_wait(t)
    monkeypatch.delenv("XC_HOST_CHUNKS")
    ref = xcorr.correlate(mode, torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(),
                          method=method).cpu().numpy()
    assert rel_to_max(ho, ref) <= 1e-5


def test_release_waits_for_calls_in_flight():
    mode, method, left, right = make(PROBLEMS[3])
    hl, _tl = pinned(left)
    hr, _tr = pinned(right)
    outs = [pinned(np.full(out_shape(mode, left, right), np.nan, np.float32)) for _ in range(2)]
    for ho, _ in outs:
        xcorr.correlate_host_async(mode, hl, hr, ho, method=method)
    xcorr.lib().xc_release_thread_cache()
    ref = xcorr.correlate_host(mode, left, right, method=method)
    for ho, _ in outs:
        assert rel_to_max(ho, ref) <= 4e-6


def test_synchronous_calls_between_stream_calls():
    """A synchronous host-buffer call in the middle of a stream (default
    stream, as the Python helpers pass it) completes the calls before it as
    needed and leaves the later ones correct."""
    mode, method, left, right = make(PROBLEMS[1])
    hl, _tl = pinned(left)
    hr, _tr = pinned(right)
    ref = xcorr.correlate_host(mode, left, right, method=method)
    outs = [pinned(np.full(out_shape(mode, left, right), np.nan, np.float32)) for _ in range(3)]
    t0 = xcorr.correlate_host_async(mode, hl, hr, outs[0][0], method=method)
    mid = xcorr.correlate_host(mode, left, right, method="fft")
    t1 = xcorr.correlate_host_async(mode, hl, hr, outs[1][0], method=method)
    t2 = xcorr.correlate_host_async(mode, hl, hr, outs[2][0], method=method)
    for t in (t0, t1, t2):
        xcorr.host_wait(t)
    for ho, _ in outs:
        assert rel_to_max(ho, ref) <= 1e-6
    assert rel_to_max(mid, ref) <= 1e-5
