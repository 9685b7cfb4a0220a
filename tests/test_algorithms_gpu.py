"""Every selector candidate (xc_algorithm: a method and one of its tiles) run
explicitly through xc_correlate_algo, in every mode, against the oracle; and
xc_time_algorithm, which the selector's timings come from, leaves the same
result in the output."""
import ctypes

import numpy as np
import pytest

from helpers import rel_to_max, seeded
from oracle import oracle

import xcorr
from xcorr import selector

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    ("one_to_one", 1, 1, (37, 45), (30, 21)),
    ("one_to_many", 1, 9, (70, 64), (33, 48)),
    ("n_to_mn", 2, 6, (40, 40), (40, 40)),
    ("n_to_m", 3, 5, (52, 29), (17, 60)),
]


@pytest.mark.parametrize("name", selector.ALGO_NAMES)
@pytest.mark.parametrize("mode,n_l,n_r,ls,rs", CASES)
def test_candidate_matches_oracle(name, mode, n_l, n_r, ls, rs):
    left = seeded((n_l,) + ls, 71, "signed")
    right = seeded((n_r,) + rs, 72, "signed")
    out = xcorr.correlate(mode, torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda(), method=name)
    torch.cuda.synchronize()
    exact = oracle.run_mode(mode, left, right, dtype="f32acc64", threads=8)
    assert rel_to_max(out.cpu().numpy(), exact) <= 1e-5, name


@pytest.mark.parametrize("name", ["direct:3", "fft", "tc_bf16x3:32"])
def test_time_algorithm_leaves_the_result(name):
    mode, n_l, n_r, ls, rs = CASES[1]
    left = torch.from_numpy(seeded((n_l,) + ls, 73)).cuda()
    right = torch.from_numpy(seeded((n_r,) + rs, 74)).cuda()
    out = torch.full((xcorr.output_count(mode, n_l, n_r), ls[0] + rs[0] - 1, ls[1] + rs[1] - 1), float("nan"),
                     device="cuda")
    ms = selector.time_algo(mode, left, right, out, name, reps=2)
    assert ms > 0.0
    ref = xcorr.correlate(mode, left, right, method=name)
    torch.cuda.synchronize()
    assert np.isfinite(out.cpu().numpy()).all()
    assert rel_to_max(out.cpu().numpy(), ref.cpu().numpy()) <= 1e-6


def test_time_algorithm_rejects_auto_and_zero_reps():
    L = xcorr.lib()
    ms = ctypes.c_double()
    dummy = ctypes.c_void_p(256)
    s = xcorr.size2(8, 8)
    assert L.xc_time_algorithm(0, 0, xcorr.Algo(xcorr.METHODS["auto"], 0), dummy, s, 1, dummy, s, 1, dummy, None, 0,
                               1, None, ctypes.byref(ms)) == 1
    assert L.xc_time_algorithm(0, 0, xcorr.Algo(xcorr.METHODS["direct"], 1), dummy, s, 1, dummy, s, 1, dummy, None,
                               0, 0, None, ctypes.byref(ms)) == 1
