"""Parity of the CUDA paths with the oracle and the reference's golden vectors.

Tolerances (max|out - oracle64| / max|oracle64| per output matrix):
  FP32 direct / FFT path : 1e-5 (the accuracy gate of the metric);
                           2e-6 against the reference's FP32-level golden files
                           is not required: those files carry FP32 error themselves,
                           so the bound there is 1e-5 as well.
  FP64 direct path       : 1e-12 (FP64-exact golden files and oracle).
  FP64 FFT path          : 1e-10.
"""
import numpy as np
import pytest

from helpers import FP64_EXACT, VALID, golden_case, rel_to_max, scipy_cases, seeded
from oracle import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import xcorr  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def device():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    xcorr.check(xcorr.lib().xc_device_check(0))
    yield
    torch.cuda.synchronize()


def dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def run(mode, left, right, method, dtype=torch.float32):
    out = xcorr.correlate(mode, dev(left, dtype), dev(right, dtype), method=method)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("method", ["direct", "fft"])
@pytest.mark.parametrize("name", VALID)
def test_golden_fp32(name, method):
    mode, left, right, valid = golden_case(name)
    out = run(mode, left, right, method)
    assert out.shape == valid.shape
    assert rel_to_max(out, valid) <= 1e-5


@pytest.mark.parametrize("name", sorted(FP64_EXACT))
def test_golden_fp64_direct(name):
    mode, left, right, valid = golden_case(name)
    out = run(mode, left, right, "direct", torch.float64)
    assert rel_to_max(out, valid) <= 1e-12


@pytest.mark.parametrize("name", sorted(FP64_EXACT))
def test_golden_fp64_fft(name):
    mode, left, right, valid = golden_case(name)
    out = run(mode, left, right, "fft", torch.float64)
    assert rel_to_max(out, valid) <= 1e-10


@pytest.mark.parametrize("method", ["direct", "fft"])
@pytest.mark.parametrize("case", range(12))
def test_reference_scipy_cases(case, method):
    """Odd sizes, 1xN strips and unequal left/right sizes."""
    mode, left, right, ref = scipy_cases()[case]
    out = run(mode, left, right, method)
    assert out.shape == ref.shape
    assert rel_to_max(out, ref) <= 1e-5
    out64 = run(mode, left, right, method, torch.float64)
    assert rel_to_max(out64, ref) <= (1e-12 if method == "direct" else 1e-10)


# Seeded sizes around the kernel's tile edges (32 x 64 shifts, 128-column
# chunks), including widths that are not a multiple of 4 (cp.async loader).
SHAPES = [
    ("one_to_one", 1, 1, (1, 1), (1, 1)),
    ("one_to_one", 1, 1, (33, 65), (33, 65)),
    ("one_to_one", 1, 1, (130, 131), (7, 200)),
    ("one_to_many", 1, 9, (64, 64), (64, 64)),
    ("one_to_many", 1, 5, (37, 150), (61, 3)),
    ("n_to_mn", 3, 9, (29, 29), (29, 29)),
    ("n_to_m", 2, 5, (48, 20), (16, 52)),
    ("n_to_m", 3, 3, (70, 1), (5, 1)),
]


@pytest.mark.parametrize("dist", ["uniform", "normal"])
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[0]}-{s[3]}-{s[4]}" for s in SHAPES])
def test_seeded_shapes_direct_and_fft(shape, dist):
    mode, n, m, ls, rs = shape
    left = seeded((n,) + ls, 100 + n, dist)
    right = seeded((m,) + rs, 200 + m, dist)
    ref = oracle.run_mode(mode, left, right, dtype="f32acc64", threads=8)
    for method in ("direct", "fft"):
        out = run(mode, left, right, method)
        assert out.shape == ref.shape
        assert rel_to_max(out, ref) <= 1e-5, method


def test_direct_fp32_accuracy_at_256_one_to_many():
    """Long overlaps (256x256) stay under the 1e-5 gate thanks to the flushed
    partial sums; 4 right matrices of the bench shape."""
    left = seeded((1, 256, 256), 2)
    right = seeded((4, 256, 256), 3)
    ref = oracle.run_mode("one_to_many", left, right, dtype="f32acc64", threads=8)
    out = run("one_to_many", left, right, "direct")
    assert rel_to_max(out, ref) <= 1e-5


def test_direct_loaders_agree():
    """TMA loader and cp.async loader give the same sums on aligned widths."""
    left = seeded((2, 40, 64), 7, "normal")
    right = seeded((4, 24, 32), 8, "normal")
    ref = oracle.run_mode("n_to_mn", left, right, dtype="f32acc64")
    out = run("n_to_mn", left, right, "direct")
    assert rel_to_max(out, ref) <= 1e-5


def test_fft_raw_output_matches_reference_normalisation():
    """normalize=0 returns the raw circular result; the reference's host
    normalisation of it equals the full correlation."""
    left = seeded((1, 20, 20), 11)
    right = seeded((3, 20, 20), 12)
    plan = xcorr.FftPlan("one_to_many", "f32", (20, 20), 1, (20, 20), 3)
    assert plan.pad == (40, 40)
    ws = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device="cuda")
    raw = torch.empty((3, 40, 40), dtype=torch.float32, device="cuda")
    plan.execute(dev(left), dev(right), raw, ws, normalize=False)
    torch.cuda.synchronize()
    norm = oracle.normalize_fft(raw.cpu().numpy())
    ref = oracle.run_mode("one_to_many", left, right)
    assert rel_to_max(norm, ref) <= 1e-5
    plan.close()


def test_host_buffer_entry_point():
    left = seeded((2, 30, 30), 21)
    right = seeded((3, 30, 30), 22)
    ref = oracle.run_mode("n_to_m", left, right)
    for method in ("direct", "fft"):
        out = xcorr.correlate_host("n_to_m", left, right, method=method)
        assert rel_to_max(out, ref) <= 1e-5
    out64 = xcorr.correlate_host("n_to_m", left.astype(np.float64), right.astype(np.float64))
    assert rel_to_max(out64, oracle.run_mode("n_to_m", left.astype(np.float64), right.astype(np.float64),
                                             dtype="f64")) <= 1e-12


def test_reference_launchers():
    """Drop-ins for run_ccn_shuffle* launchers (src/kernels.cuh)."""
    import ctypes
    L = xcorr.lib()
    left = dev(seeded((1, 17, 17), 31))
    right = dev(seeded((6, 17, 17), 32))
    out = torch.zeros((6, 33, 33), device="cuda")
    ms, ss = xcorr.size2(17, 17), xcorr.size2(33, 33)
    st = torch.cuda.current_stream().cuda_stream
    xcorr.check(L.xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f32(
        left.data_ptr(), right.data_ptr(), out.data_ptr(), ms, ss, 6, 8, 4, 4, 4, st))
    torch.cuda.synchronize()
    ref = oracle.run_mode("one_to_many", left.cpu().numpy(), right.cpu().numpy())
    assert rel_to_max(out.cpu().numpy(), ref) <= 1e-5
    # the reference's limits are enforced
    assert L.xc_run_ccn_shuffle_f32(left.data_ptr(), right.data_ptr(), out.data_ptr(), ms, ss, 33, st) == 1
    assert L.xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f32(
        left.data_ptr(), right.data_ptr(), out.data_ptr(), ms, ss, 6, 8, 5, 4, 4, st) == 1
    # n_to_m launcher: output l*M + r
    lefts = dev(seeded((2, 9, 9), 33))
    rights = dev(seeded((3, 9, 9), 34))
    o2 = torch.zeros((6, 17, 17), device="cuda")
    xcorr.check(L.xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_f32(
        lefts.data_ptr(), rights.data_ptr(), o2.data_ptr(), xcorr.size2(9, 9), xcorr.size2(17, 17), 2, 3, 8, 2, 2, 2,
        2, st))
    torch.cuda.synchronize()
    ref2 = oracle.run_mode("n_to_m", lefts.cpu().numpy(), rights.cpu().numpy())
    assert rel_to_max(o2.cpu().numpy(), ref2) <= 1e-5


# (launcher, mode, n_left, n_right, extra arguments after search_size, adds into out)
# Extra arguments follow src/kernels.cuh: counts, warps per block, tile
# arguments, then max_rows_per_thread and the distribution for the
# work-distribution launchers (1 = rectangle, 2 = triangle, 0 = none).
MORE_LAUNCHERS = [
    ("xc_run_ccn_shuffle_work_distribution", "one_to_one", 1, 1, (8, 5, 2), True),
    ("xc_run_ccn_shuffle_work_distribution", "one_to_one", 1, 1, (4, 0, 0), True),
    ("xc_run_ccn_shuffle_multimat_right_work_distribution", "one_to_many", 1, 5, (5, 8, 4, 7, 1), True),
    ("xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution", "n_to_m", 3, 4, (3, 4, 8, 2, 2, 6, 2), True),
    ("xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem", "n_to_m", 2, 3, (2, 3, 8, 4, 4, 3, 1),
     True),
    ("xc_run_ccn_shuffle_multirow_right", "one_to_one", 1, 1, (8, 4), False),
    ("xc_run_ccn_shuffle_multirow_both", "one_to_one", 1, 1, (8, 4, 2), False),
    ("xc_run_ccn_shuffle_multirow_both_local_mem", "one_to_one", 1, 1, (8, 8, 4), False),
    ("xc_run_ccn_shuffle_multirow_right_multimat_right", "one_to_many", 1, 6, (6, 8, 2, 3), False),
]


@pytest.mark.parametrize("side", [23, 96])
@pytest.mark.parametrize("suffix", ["f32", "f64"])
@pytest.mark.parametrize("case", MORE_LAUNCHERS, ids=lambda c: c[0][len("xc_run_ccn_shuffle_"):] + "_" + c[1])
def test_reference_launchers_work_distribution_and_multirow(case, suffix, side):
    """The work-distribution, multirow and multirow-multimat drop-ins
    (src/kernels.cuh:75-281) against the oracle.  The work-distribution ones
    add into `out`, as the reference's atomic kernels do: the output starts at
    1.0 here and must end at 1.0 plus the correlation.  At 23x23 the plain
    kernel's tiles leave the GPU nearly empty, so its rows are split over
    CTAs (red.global.add); at 96x96 with 5-6 partners too."""
    name, mode, n, m, extra, adds = case
    dt = torch.float32 if suffix == "f32" else torch.float64
    npdt = np.float32 if suffix == "f32" else np.float64
    L = xcorr.lib()
    left = seeded((n, side, side), 60 + side, dtype=npdt)
    right = seeded((m, side, side), 61 + side, dtype=npdt)
    n_out = xcorr.output_count(mode, n, m)
    base = 1.0 if adds else float("nan")
    out = torch.full((n_out, 2 * side - 1, 2 * side - 1), base, dtype=dt, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    ms, ss = xcorr.size2(side, side), xcorr.size2(2 * side - 1, 2 * side - 1)
    fn = getattr(L, f"{name}_{suffix}")
    d_left, d_right = dev(left, dt), dev(right, dt)  # held until the kernel has run
    xcorr.check(fn(d_left.data_ptr(), d_right.data_ptr(), out.data_ptr(), ms, ss, *extra, st))
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64) - (1.0 if adds else 0.0)
    ref = oracle.run_mode(mode, left, right, dtype="f32acc64" if suffix == "f32" else "f64", threads=8)
    assert rel_to_max(got, ref) <= (1e-5 if suffix == "f32" else 1e-12)


def test_reference_launcher_limits():
    """The reference's argument checks (src/naive_shuffle*.cu launchers;
    release limits, CMakeLists.txt:16-43) return XC_ERR_INVALID_ARGUMENT."""
    L = xcorr.lib()
    p = 16  # never dereferenced: every call below is rejected first
    ms, ss = xcorr.size2(8, 8), xcorr.size2(15, 15)
    assert L.xc_run_ccn_shuffle_work_distribution_f32(p, p, p, ms, ss, 33, 4, 1, None) == 1  # warps > 32
    assert L.xc_run_ccn_shuffle_work_distribution_f32(p, p, p, ms, ss, 8, 0, 2, None) == 1  # triangle, 0 rows
    assert L.xc_run_ccn_shuffle_work_distribution_f32(p, p, p, ms, ss, 8, 4, 3, None) == 1  # unknown distribution
    assert L.xc_run_ccn_shuffle_multimat_right_work_distribution_f32(p, p, p, ms, ss, 4, 8, 9, 4, 1, None) == 1
    assert L.xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_f64(p, p, p, ms, ss, 2, 2, 8, 5, 1, 4, 1,
                                                                            None) == 1
    assert L.xc_run_ccn_shuffle_multirow_right_f32(p, p, p, ms, ss, 8, 9, None) == 1
    assert L.xc_run_ccn_shuffle_multirow_both_f32(p, p, p, ms, ss, 8, 4, 5, None) == 1
    assert L.xc_run_ccn_shuffle_multirow_both_local_mem_f64(p, p, p, ms, ss, 8, 9, 2, None) == 1
    assert L.xc_run_ccn_shuffle_multirow_right_multimat_right_f32(p, p, p, ms, ss, 3, 8, 5, 2, None) == 1
    assert L.xc_run_ccn_shuffle_multirow_right_multimat_right_f32(p, p, p, ms, ss, 3, 8, 2, 0, None) == 1
    assert L.xc_run_ccn_shuffle_multirow_right_f32(p, p, p, ms, xcorr.size2(16, 15), 8, 2, None) == 1  # search size


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_fft_transform_side_1024_or_more_small_right(dtype):
    """Transform sides of 1024 or more normalise in FP64: a 1000x1000 left
    with 40x40 rights (1039-point sides padded to a smooth size) against the
    oracle, in FP32 and FP64."""
    npdt = np.float32 if dtype == "f32" else np.float64
    tdt = torch.float32 if dtype == "f32" else torch.float64
    left = seeded((1, 1000, 1000), 71, dtype=npdt)
    right = seeded((3, 40, 40), 72, "signed", dtype=npdt)
    got = run("one_to_many", left, right, "fft", tdt)
    ref = oracle.run_mode("one_to_many", left, right, dtype="f32acc64" if dtype == "f32" else "f64", threads=8)
    assert rel_to_max(got, ref) <= (1e-5 if dtype == "f32" else 1e-10)


def test_fft_equal_sides_1024_against_fp64():
    """1024x1024 left and two 1024x1024 rights (2048x2048 transforms), FP32
    FFT: every output against the library's FP64 FFT of the same inputs, and
    against FP64 sums on the CPU at 48 sampled shifts per output (the centre
    shift, the longest sum, included)."""
    left = seeded((1, 1024, 1024), 73)
    right = seeded((2, 1024, 1024), 74)
    got = run("one_to_many", left, right, "fft")
    ref = run("one_to_many", left.astype(np.float64), right.astype(np.float64), "fft", torch.float64)
    assert rel_to_max(got, ref) <= 1e-5
    rng = np.random.default_rng(75)
    L = left[0].astype(np.float64)
    for k in range(2):
        R = right[k].astype(np.float64)
        scale = np.abs(ref[k]).max()
        oys = np.concatenate([[1023], rng.integers(0, 2047, 47)])
        oxs = np.concatenate([[1023], rng.integers(0, 2047, 47)])
        for oy, ox in zip(oys, oxs):
            dy, dx = int(oy) - 1023, int(ox) - 1023
            y0, y1 = max(0, -dy), min(1024, 1024 - dy)
            x0, x1 = max(0, -dx), min(1024, 1024 - dx)
            exact = np.sum(L[y0 + dy:y1 + dy, x0 + dx:x1 + dx] * R[y0:y1, x0:x1])
            assert abs(got[k][oy, ox] - exact) / scale <= 1e-5
            assert abs(ref[k][oy, ox] - exact) / scale <= 1e-10


def test_fft_glue_launchers():
    """hadamard_original / hadamard_n_to_m_over_output / scatter / normalize drop-ins."""
    L = xcorr.lib()
    st = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(41)
    ref = (rng.standard_normal((4, 5)) + 1j * rng.standard_normal((4, 5))).astype(np.complex64)
    deformed = (rng.standard_normal((3, 4, 5)) + 1j * rng.standard_normal((3, 4, 5))).astype(np.complex64)
    d_ref = torch.as_tensor(ref).cuda()
    d_def = torch.as_tensor(deformed).cuda()
    xcorr.check(L.xc_run_hadamard_original_c64(d_ref.data_ptr(), d_def.data_ptr(), xcorr.size2(4, 5), 1, 3, 128, st))
    torch.cuda.synchronize()
    np.testing.assert_allclose(d_def.cpu().numpy(), ref[None] * np.conj(deformed), rtol=1e-6, atol=1e-6)

    lt = (rng.standard_normal((2, 6)) + 1j * rng.standard_normal((2, 6))).astype(np.complex64)
    rt = (rng.standard_normal((3, 6)) + 1j * rng.standard_normal((3, 6))).astype(np.complex64)
    o = torch.zeros((2, 3, 6), dtype=torch.complex64, device="cuda")
    d_lt = torch.as_tensor(lt).cuda()
    d_rt = torch.as_tensor(rt).cuda()
    xcorr.check(L.xc_run_hadamard_n_to_m_over_output_c64(d_lt.data_ptr(), d_rt.data_ptr(), o.data_ptr(),
                                                         xcorr.size2(2, 3), 2, 3, 256, 1, st))
    torch.cuda.synchronize()
    np.testing.assert_allclose(o.cpu().numpy(), lt[:, None, :] * np.conj(rt[None, :, :]), rtol=1e-6, atol=1e-6)

    src = seeded((2, 3, 5), 42)
    dst = torch.full((2, 6, 10), 7.0, device="cuda")
    xcorr.check(L.xc_run_scatter_f32(dev(src).data_ptr(), dst.data_ptr(), xcorr.size2(3, 5), 2, xcorr.size2(6, 10),
                                     xcorr.size2(1, 2), 256, 10, st))
    torch.cuda.synchronize()
    exp = np.zeros((2, 6, 10), np.float32)
    exp[:, 1:4, 2:7] = src
    np.testing.assert_array_equal(dst.cpu().numpy(), exp)

    raw = seeded((2, 8, 6), 43, "normal")
    norm = torch.zeros((2, 7, 5), device="cuda")
    xcorr.check(L.xc_normalize_fft_results_f32(dev(raw).data_ptr(), norm.data_ptr(), xcorr.size2(8, 6), 2, st))
    torch.cuda.synchronize()
    np.testing.assert_allclose(norm.cpu().numpy(), oracle.normalize_fft(raw), rtol=1e-6, atol=1e-7)


def test_errors_are_reported_not_fatal():
    with pytest.raises(xcorr.XcError) as e:
        xcorr.correlate("n_to_mn", dev(seeded((3, 4, 4), 1)), dev(seeded((4, 4, 4), 2)))
    assert e.value.status == 1
    # the context is still usable
    out = run("one_to_one", seeded((1, 4, 4), 1), seeded((1, 4, 4), 2), "direct")
    assert out.shape == (1, 7, 7)


@pytest.mark.parametrize("mode,n_l,n_r,side,chunks", [
    ("one_to_many", 1, 7, 120, 2),   # 7 partners: chunks of 4, 3
    ("n_to_mn", 3, 15, 64, 3),       # 5 partners of each left: chunks of 2, 2, 1
    ("n_to_m", 5, 3, 64, 4),         # 5 lefts: chunks of 2, 2, 1
    ("n_to_m", 5, 3, 64, 1),
])
def test_host_buffer_entry_point_pipelined(mode, n_l, n_r, side, chunks, monkeypatch):
    """The chunked copy-in / correlate / copy-out pipeline (XC_HOST_CHUNKS
    fixes the chunk count): every chunk must land where the one-shot device
    call puts it."""
    monkeypatch.setenv("XC_HOST_CHUNKS", str(chunks))
    left = seeded((n_l, side, side), 41)
    right = seeded((n_r, side, side), 42)
    for method in ("direct", "tc_bf16x3"):
        out = xcorr.correlate_host(mode, left, right, method=method)
        ref = xcorr.correlate(mode, dev(left), dev(right), method=method).cpu().numpy()
        # a chunk holds fewer partners, so a kernel may pick another tile shape
        # (and the split path other means): same products, possibly another order
        assert rel_to_max(out, ref) <= 1e-5


@pytest.mark.parametrize("mode,n_l,n_r,side,bands", [
    ("one_to_many", 1, 9, 96, 3),
    ("n_to_mn", 2, 6, 80, 4),
    ("n_to_m", 3, 4, 64, 2),
    ("one_to_one", 1, 1, 200, 8),
])
@pytest.mark.parametrize("method", ["tc_bf16x3", "tc_tf32x3"])
def test_host_buffer_entry_point_banded(mode, n_l, n_r, side, bands, method, monkeypatch):
    """Split tensor-core path through the host-buffer call with the output
    copied out in row bands while the kernel runs (XC_HOST_BANDS fixes the
    band count): every band's rows must match the one-shot device call."""
    monkeypatch.setenv("XC_HOST_BANDS", str(bands))
    monkeypatch.delenv("XC_HOST_CHUNKS", raising=False)
    left = seeded((n_l, side, side), 51)
    right = seeded((n_r, side - 7, side + 5), 52)
    out = xcorr.correlate_host(mode, left, right, method=method)
    ref = xcorr.correlate(mode, dev(left), dev(right), method=method).cpu().numpy()
    # a banded launch cuts each band's left rows into pieces of its own (other
    # drain points, another order of the reductions into the output): the
    # same products summed in another order, so the two runs agree to a few
    # FP32 roundings of the partial sums, and each meets the 1e-5 gate
    assert rel_to_max(out, ref) <= 4e-6
    exact = oracle.run_mode(mode, left, right, dtype="f32acc64", threads=8)
    assert rel_to_max(out, exact) <= 1e-5
    assert rel_to_max(ref, exact) <= 1e-5
