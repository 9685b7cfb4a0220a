"""Failure detection without a GPU fault: a bounded device-side wait that
expires is reported to the host as XC_ERR_TIMEOUT and leaves the context
usable."""
import numpy as np
import pytest

from helpers import rel_to_max, seeded
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import xcorr  # noqa: E402


def test_expired_wait_is_reported_and_context_survives():
    L = xcorr.lib()
    st = torch.cuda.current_stream().cuda_stream
    assert L.xc_check_device(st) == 0
    xcorr.check(L.xc_debug_expire_wait(2000, st))
    assert L.xc_check_device(st) == 6  # XC_ERR_TIMEOUT
    assert b"bounded device wait expired" in L.xc_last_error()
    # the record is cleared and the context still computes correct results
    assert L.xc_check_device(st) == 0
    left, right = seeded((1, 20, 20), 1), seeded((3, 20, 20), 2)
    out = xcorr.correlate("one_to_many", torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(),
                          method="tc_bf16x3")
    assert L.xc_check_device(st) == 0
    assert rel_to_max(out.cpu().numpy(), oracle.run_mode("one_to_many", left, right)) <= 1e-5


def test_invalid_hook_argument():
    assert xcorr.lib().xc_debug_expire_wait(0, None) == 1
