"""xc_correlate_tc_noalloc: the split-BF16 correlation for callers that may not
allocate device memory (hosts that own the memory budget or pool, and
latency-critical loops where cudaMalloc/cudaFree may block or synchronise).

It works in one fixed file-scope device array instead of a caller workspace,
so these tests call it twice in a row through the C ABI and compare each
result with the ordinary workspace entry point (xc_correlate with
XC_METHOD_TC_BF16X3) and with the CPU oracle (FP64 accumulation), within the
1e-5 relative tolerance the other parity tests use.  The second call uses a
different shape, so stale contents of the shared array from the first call
must not matter.  A further test checks the entry point's promise itself:
after a warm-up call, repeated calls leave the device's free memory where it
was.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_to_max, seeded
from oracle import oracle

import xcorr

# (mode, n_left, n_right, left shape, right shape, distribution)
CALLS = [
    ("one_to_many", 1, 9, (40, 48), (40, 48), "uniform"),
    ("n_to_m", 2, 5, (30, 66), (21, 17), "signed"),
]


def noalloc(mode, left, right, out, stream):
    n, hl, wl = left.shape
    m, hr, wr = right.shape
    return xcorr.lib().xc_correlate_tc_noalloc(xcorr.MODES[mode], left.data_ptr(), xcorr.size2(hl, wl), n,
                                               right.data_ptr(), xcorr.size2(hr, wr), m, out.data_ptr(), stream)


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    stream = torch.cuda.current_stream().cuda_stream
    for i, (mode, n, m, ls, rs, dist) in enumerate(CALLS):
        left = torch.as_tensor(seeded((n,) + ls, 500 + i, dist)).cuda()
        right = torch.as_tensor(seeded((m,) + rs, 600 + i, dist)).cuda()
        n_out = xcorr.output_count(mode, n, m)
        out = torch.full((n_out, ls[0] + rs[0] - 1, ls[1] + rs[1] - 1), float("nan"), device="cuda")
        xcorr.check(noalloc(mode, left, right, out, stream))
        ref = xcorr.correlate(mode, left, right, method="tc_bf16x3")
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_to_max(got, ref.cpu().numpy()) <= 1e-5, f"call {i}"
        exact = oracle.run_mode(mode, left.cpu().numpy(), right.cpu().numpy(), dtype="f32acc64", threads=8)
        assert rel_to_max(got, exact) <= 1e-5, f"call {i} against the oracle"


@pytest.mark.gpu
def test_noalloc_calls_leave_free_device_memory_unchanged():
    """The array is part of the loaded module; no call may take device memory
    beyond it.  The warm-up call may load the module; after it, free memory
    (cudaMemGetInfo) must not drop over repeated calls.  The inputs and
    outputs are allocated before the first reading."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    stream = torch.cuda.current_stream().cuda_stream
    mode, n, m, ls, rs, dist = CALLS[0]
    left = torch.as_tensor(seeded((n,) + ls, 700, dist)).cuda()
    right = torch.as_tensor(seeded((m,) + rs, 701, dist)).cuda()
    out = torch.empty((xcorr.output_count(mode, n, m), ls[0] + rs[0] - 1, ls[1] + rs[1] - 1), device="cuda")
    xcorr.check(noalloc(mode, left, right, out, stream))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        xcorr.check(noalloc(mode, left, right, out, stream))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, f"free device memory dropped by {free0 - free1} bytes"


def test_noalloc_rejects_problems_larger_than_its_array():
    """Needs no GPU: the size check runs before any CUDA call."""
    L = xcorr.lib()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the call is rejected first
    # 1 left + 1024 right 256x256 matrices need ~800 MB of scratch > 64 MiB
    st = L.xc_correlate_tc_noalloc(xcorr.MODES["one_to_many"], dummy, xcorr.size2(256, 256), 1, dummy,
                                   xcorr.size2(256, 256), 1024, dummy, None)
    assert st == 5  # XC_ERR_WORKSPACE
    msg = L.xc_last_error().decode()
    assert "scratch" in msg and str(64 * 1024 * 1024) in msg
