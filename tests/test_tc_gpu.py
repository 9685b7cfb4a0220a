"""Split-BF16 and split-TF32 tensor-core paths (tcgen05) against the oracle.

Tolerance: max|out - oracle64| / max|oracle64| <= 1e-5 per output matrix,
the accuracy gate of the headline metric.
"""
import numpy as np
import pytest

from helpers import VALID, golden_case, rel_to_max, seeded
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import xcorr  # noqa: E402


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).cuda()


TC_METHODS = ["tc_bf16x3", "tc_tf32x3"]


def run_tc(mode, left, right, method="tc_bf16x3"):
    out = xcorr.correlate(mode, dev(left), dev(right), method=method)
    torch.cuda.synchronize()
    xcorr.check(xcorr.lib().xc_device_check(0))
    return out.cpu().numpy()


TC_SHAPES = [
    # (mode, n_left, n_right, left, right, dist) -- partners per tile P = 1, 2, 4 use
    # one TMA box per partner; P >= 8 one box per row shift
    ("one_to_one", 1, 1, (17, 17), (17, 17), "uniform"),
    ("one_to_many", 1, 2, (20, 24), (20, 24), "normal"),
    ("one_to_many", 1, 4, (33, 40), (12, 9), "uniform"),
    ("n_to_mn", 2, 6, (19, 19), (19, 19), "normal"),
    ("one_to_many", 1, 9, (64, 64), (64, 64), "uniform"),
    ("n_to_m", 2, 16, (30, 70), (30, 66), "signed"),
    ("one_to_many", 1, 64, (40, 48), (40, 48), "uniform"),
    # narrow left rows under wide shift ranges: windowed MMAs over part of the
    # B rows; right widths that leave empty K-steps in the last 64-column chunk
    ("one_to_many", 1, 3, (12, 40), (10, 200), "uniform"),
    ("one_to_one", 1, 1, (9, 100), (7, 250), "normal"),
    ("n_to_m", 2, 3, (16, 256), (12, 256), "signed"),
    # partner groups of 8, 32 and 256 (row shifts per B tile 32, 8, 1), three
    # shift tiles (one item holds a single tile), one shift tile
    ("one_to_many", 1, 7, (24, 24), (20, 28), "uniform"),
    ("one_to_many", 1, 20, (18, 30), (16, 22), "normal"),
    ("one_to_many", 1, 130, (9, 11), (8, 13), "uniform"),
    ("n_to_mn", 2, 10, (12, 180), (10, 150), "signed"),
    ("one_to_one", 1, 1, (40, 60), (30, 50), "uniform"),
    # beyond 512 output columns (x-parts of 512 shifts) and 256 right columns
    # (k-parts of 256 columns), including a small template on a wide left
    ("one_to_many", 1, 3, (30, 700), (20, 300), "uniform"),
    ("one_to_one", 1, 1, (8, 300), (8, 300), "normal"),
    ("n_to_m", 2, 2, (12, 520), (10, 260), "signed"),
    ("one_to_many", 1, 9, (40, 1100), (16, 16), "uniform"),
    ("one_to_one", 1, 1, (6, 40), (5, 600), "normal"),
]


@pytest.mark.parametrize("method", TC_METHODS)
@pytest.mark.parametrize("shape", TC_SHAPES, ids=[f"{s[0]}-{s[1]}x{s[2]}-{s[3]}-{s[4]}" for s in TC_SHAPES])
def test_tc_matches_oracle(shape, method):
    mode, n, m, ls, rs, dist = shape
    left = seeded((n,) + ls, 300 + n, dist)
    right = seeded((m,) + rs, 400 + m, dist)
    ref = oracle.run_mode(mode, left, right, dtype="f32acc64", threads=8)
    out = run_tc(mode, left, right, method)
    assert out.shape == ref.shape
    assert rel_to_max(out, ref) <= 1e-5


@pytest.mark.parametrize("method", TC_METHODS)
@pytest.mark.parametrize("name", [v for v in VALID if "_10_10_" in v or "_64_64_" in v])
def test_tc_golden(name, method):
    mode, left, right, valid = golden_case(name)
    out = run_tc(mode, left.astype(np.float32), right.astype(np.float32), method)
    assert rel_to_max(out, valid) <= 1e-5


@pytest.mark.parametrize("method", TC_METHODS)
def test_tc_bench_shape_accuracy(method):
    """The benchmark's shape (256x256, 64 right matrices) on 8 of them."""
    left = seeded((1, 256, 256), 2)
    right = seeded((8, 256, 256), 3)
    ref = oracle.run_mode("one_to_many", left, right, dtype="f32acc64", threads=16)
    out = run_tc("one_to_many", left, right, method)
    assert rel_to_max(out, ref) <= 1e-5


@pytest.mark.parametrize("method", TC_METHODS)
def test_tc_rejects_unsupported_sizes(method):
    """Wl + Wr above 6400: the mean-correction kernel's staged rows would
    pass its shared-memory budget."""
    with pytest.raises(xcorr.XcError) as e:
        xcorr.correlate("one_to_one", dev(seeded((1, 2, 4000), 1)), dev(seeded((1, 2, 2500), 2)), method=method)
    assert e.value.status == 4


def test_tf32_more_accurate_than_bf16_on_zero_mean_data():
    """TF32 operands keep ~21 bits against BF16's ~16: on zero-mean data,
    where the mean shift does not help, the TF32x3 error is the smaller."""
    left = seeded((1, 96, 96), 7, "normal")
    right = seeded((4, 96, 96), 8, "normal")
    ref = oracle.run_mode("one_to_many", left, right, dtype="f32acc64", threads=16)
    e_bf = rel_to_max(run_tc("one_to_many", left, right, "tc_bf16x3"), ref)
    e_tf = rel_to_max(run_tc("one_to_many", left, right, "tc_tf32x3"), ref)
    assert e_tf <= 1e-5 and e_tf < e_bf
