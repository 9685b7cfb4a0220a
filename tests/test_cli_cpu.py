"""The `cross` CLI on the host: algorithm registry, cpu_* algorithms, the
validate and input commands, argument errors and exit codes
(src/main.cpp:465-683).  No GPU needed."""
import os
import subprocess

import numpy as np
import pytest

from helpers import DATA, FP64_EXACT, golden_paths
from oracle import oracle

import xcorr

CROSS = xcorr.CLI_PATH

# get_algorithms (src/main.cpp:361-411), sorted like `cross list`
REFERENCE_ALGS = sorted("""cpu_one_to_one cpu_one_to_many cpu_n_to_mn cpu_n_to_m nai_orig_one_to_one
nai_orig_one_to_many nai_orig_n_to_mn nai_orig_n_to_m nai_shuffle_one_to_one nai_shuffle_work_distribution_one_to_one
nai_shuffle_multimat_right_one_to_one nai_shuffle_multimat_right_one_to_many
nai_shuffle_multimat_right_work_distribution_one_to_one nai_shuffle_multimat_right_work_distribution_one_to_many
nai_shuffle_multimat_right_work_distribution_n_to_mn nai_shuffle_multimat_right_work_distribution_n_to_m
nai_shuffle_multimat_both_work_distribution_local_mem_n_to_m nai_shuffle_multimat_both_work_distribution_n_to_m
nai_shuffle_multirow_both_multimat_both_n_to_m nai_shuffle_multirow_right_one_to_one
nai_shuffle_multirow_both_one_to_one nai_shuffle_multirow_both_local_mem_one_to_one
nai_shuffle_multirow_right_multimat_right_one_to_one nai_shuffle_multirow_right_multimat_right_one_to_many
nai_shuffle_multirow_right_multimat_right_n_to_mn nai_shuffle_multirow_both_multimat_right_one_to_many
nai_shuffle_multirow_both_multimat_right_n_to_mn nai_warp_per_shift_one_to_one
nai_warp_per_shift_simple_indexing_one_to_one nai_warp_per_shift_work_distribution_one_to_one
nai_warp_per_shift_shared_mem_one_to_one nai_warp_per_shift_shared_mem_one_to_many nai_warp_per_shift_shared_mem_n_to_mn
nai_warp_per_shift_shared_mem_n_to_m nai_block_per_shift_one_to_one fft_orig_one_to_one fft_reduced_transfer_one_to_one
fft_orig_one_to_many fft_reduced_transfer_one_to_many fft_orig_n_to_mn fft_reduced_transfer_n_to_mn
fft_better_n_to_m""".split())


def gunzip(tmp_path, path):
    import gzip
    dst = tmp_path / os.path.basename(path)[:-3]
    dst.write_bytes(gzip.open(path).read())
    return str(dst)


def cross(*args, cwd=None):
    return subprocess.run([CROSS, *args], capture_output=True, text=True, cwd=cwd)


def test_cli_built():
    assert os.path.exists(CROSS)


def test_list_has_every_reference_algorithm():
    r = cross("list")
    assert r.returncode == 0
    names = r.stdout.split()
    assert names == sorted(names)
    assert set(REFERENCE_ALGS) <= set(names)
    assert {"tc_bf16x3_one_to_one", "tc_bf16x3_one_to_many", "tc_bf16x3_n_to_mn", "tc_bf16x3_n_to_m"} <= set(names)
    assert {"tc_tf32x3_one_to_one", "tc_tf32x3_one_to_many", "tc_tf32x3_n_to_mn", "tc_tf32x3_n_to_m"} <= set(names)


@pytest.mark.parametrize("name", ["valid_one_to_one_10_10_1_1_1_2.csv.gz", "valid_one_to_many_64_64_1_2_1_1.csv.gz",
                                  "valid_n_to_mn_10_10_2_4_1_1.csv.gz", "valid_n_to_m_10_10_4_4_1_1.csv.gz"])
def test_cpu_algorithm_with_golden_file(tmp_path, name):
    mode, lp, rp, vp = golden_paths(name)
    lp, rp, vp = gunzip(tmp_path, lp), gunzip(tmp_path, rp), gunzip(tmp_path, vp)
    out = tmp_path / "out.csv"
    r = cross("run", "-p", "-d", "double", "-v", vp, "-o", str(out), f"cpu_{mode}", lp, rp)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    exact = name in FP64_EXACT  # the other golden files carry FP32-level values
    assert lines[0] == "Max,Mean,Stddev"
    assert float(lines[1].split(",")[0]) < (1e-9 if exact else 1e-3)
    res = oracle.read_csv(str(out))
    valid = oracle.read_csv(vp)
    assert res.shape == valid.shape
    np.testing.assert_allclose(res, valid, rtol=0, atol=(1e-12 if exact else 2e-6) * np.abs(valid).max())


def test_validate_command_and_normalize(tmp_path):
    rng = np.random.default_rng(1)
    L = rng.random((7, 6))
    R = rng.random((7, 6))
    full = oracle.correlate(L, R, dtype="f64")
    P = (14, 12)
    raw = np.fft.irfft2(np.fft.rfft2(L, P) * np.conj(np.fft.rfft2(R, P)), P) * (P[0] * P[1])
    oracle.write_csv(str(tmp_path / "valid.csv"), full)
    oracle.write_csv(str(tmp_path / "raw.csv"), raw)
    r = cross("validate", "-n", "-c", "-p", str(tmp_path / "valid.csv"), str(tmp_path / "raw.csv"))
    assert r.returncode == 0, r.stderr
    out = r.stdout.strip().splitlines()
    assert out[0] == "Max,Mean,Stddev" and float(out[1].split(",")[0]) < 1e-10
    r = cross("validate", str(tmp_path / "valid.csv"), str(tmp_path / "valid.csv"))
    assert "Difference from valid values:" in r.stdout and "Max: 0" in r.stdout


def test_input_command():
    assert cross("input", "n_to_mn", "10", "10", "2", "6").stdout == "Valid\n"
    assert cross("input", "n_to_mn", "10", "10", "4", "6").stdout == "Invalid\n"
    assert cross("input", "one_to_one", "10", "10", "1", "1").stdout == "Valid\n"
    assert cross("input", "one_to_many", "0", "10", "1", "2").stdout == "Invalid\n"
    r = cross("input", "bogus", "1", "1", "1", "1")
    assert r.returncode == 1 and "Unknown algorithm type" in r.stderr


def test_exit_codes(tmp_path):
    lp = gunzip(tmp_path, os.path.join(DATA, "ina_10_10_1_1.csv.gz"))
    assert cross("run", "no_such_alg", lp, lp).returncode == 1
    assert cross("run", "--bogus", "cpu_one_to_one", lp, lp).returncode == 1
    assert cross("frobnicate").returncode == 1
    # unreadable input: failure of the load step
    assert cross("run", "cpu_one_to_one", str(tmp_path / "missing.csv"), lp).returncode == 3
    bad = tmp_path / "bad.json"
    bad.write_text('{"warps_per_thread_block": "many"}')
    assert cross("run", "--args_path", str(bad), "cpu_one_to_one", lp, lp).returncode == 0  # cpu_* read no args
    r = cross("run", "--args_path", str(bad), "nai_shuffle_one_to_one", lp, lp)
    assert r.returncode == 1 and "Invalid algorithm argument value" in r.stderr


def test_measurement_csv_for_cpu_algorithm(tmp_path):
    lp = gunzip(tmp_path, os.path.join(DATA, "ina_10_10_1_1.csv.gz"))
    rp = gunzip(tmp_path, os.path.join(DATA, "ina_10_10_1_2.csv.gz"))
    t = tmp_path / "times.csv"
    r = cross("run", "-p", "-b", "CommonSteps", "-m", "0.01", "-l", "2", "-t", str(t), "cpu_one_to_one", lp, rp)
    assert r.returncode == 0, r.stderr
    rows = t.read_text().strip().splitlines()
    assert rows[0] == ("Load,Load_iterations,Prepare,Prepare_iterations,Transfer,Transfer_iterations,Run,"
                       "Run_iterations,Finalize,Finalize_iterations,Free,Free_iterations,Store,Store_iterations")
    assert len(rows) == 3 and all(len(x.split(",")) == 14 for x in rows[1:])


def test_csv_reader_edge_cases_and_round_trip(tmp_path):
    """The CSV reader (read_header / read_data, src/matrix.hpp:94-159): CRLF
    line ends, blanks and a leading '+', malformed lines reported with the
    reference's messages (the first bad line in file order), and a round
    trip of a multi-threaded store and load through the cpu_* path."""
    good = tmp_path / "good.csv"
    good.write_bytes(b"# 2,3,1\r\n1, +2.5 ,3e-1\r\n-4,5.0,6\r\n")
    out = tmp_path / "out.csv"
    r = cross("run", "-p", "-o", str(out), "cpu_one_to_one", str(good), str(good))
    assert r.returncode == 0, r.stderr
    m = np.array([[1, 2.5, 0.3], [-4, 5, 6]])
    exp = oracle.run_mode("one_to_one", m[None], m[None], dtype="f64")[0]
    np.testing.assert_allclose(oracle.read_csv(str(out))[0], exp, rtol=1e-6)
    cases = [(b"# 2,3\n1,2,3\n4,5,6,7\n", "Line 1 is too long"),
             (b"# 2,3\n1,2\n4,5,6\n", "Line0 is too short, expected 3, got 2 values"),
             (b"# 2,3\n1,2,3\n4,x,6\n", 'Invalid value "x"'),
             (b"# 3,3\n1,2,3\n4,5,6\n", "Failed to read line 2 from csv file"),
             (b"# 2,3\n1,2,3\n4,5\n1,2\n", "Line1 is too short"),
             (b"2,3\n1,2,3\n", "Invalid file header format")]
    for k, (text, msg) in enumerate(cases):
        bad = tmp_path / f"bad{k}.csv"
        bad.write_bytes(text)
        r = cross("run", "-p", "cpu_one_to_one", str(bad), str(good))
        assert r.returncode == 3 and msg in r.stderr, (text, r.stderr)
    # a larger file: rows spread over the parser's threads; one_to_many output
    # (9 matrices) written by the formatter's threads and read back exactly
    rng = np.random.default_rng(9)
    left = rng.standard_normal((1, 40, 37)).astype(np.float32)
    right = rng.standard_normal((9, 40, 37)).astype(np.float32)
    lp, rp, op = tmp_path / "l.csv", tmp_path / "r.csv", tmp_path / "o.csv"
    for path, a in ((lp, left), (rp, right)):
        with open(path, "w") as f:
            f.write(f"# {a.shape[1]},{a.shape[2]},{a.shape[0]}\n")
            for row in a.reshape(-1, a.shape[2]):
                f.write(",".join(repr(float(v)) for v in row) + "\n")
    r = cross("run", "-p", "-o", str(op), "cpu_one_to_many", str(lp), str(rp))
    assert r.returncode == 0, r.stderr
    got = oracle.read_csv(str(op))
    ref = oracle.run_mode("one_to_many", left, right, dtype="f32")
    np.testing.assert_array_equal(got.astype(np.float32), ref.astype(np.float32))
