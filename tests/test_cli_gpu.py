"""The `cross` CLI on the GPU: every hot-path algorithm family against the
reference's golden files, raw and normalised FFT output, FP64, and the
per-algorithm timing CSV."""
import os
import subprocess

import numpy as np
import pytest

from helpers import FP64_EXACT, golden_paths, rel_to_max
from oracle import oracle

import xcorr

pytestmark = pytest.mark.gpu
CROSS = xcorr.CLI_PATH

CASES = [
    ("nai_shuffle_one_to_one", "valid_one_to_one_64_64_1_1_1_2.csv.gz"),
    ("nai_shuffle_work_distribution_one_to_one", "valid_one_to_one_128_128_1_1_1_2.csv.gz"),
    ("nai_shuffle_multimat_right_one_to_many", "valid_one_to_many_64_64_1_2_1_1.csv.gz"),
    ("nai_shuffle_multirow_both_multimat_right_one_to_many", "valid_one_to_many_10_10_1_4_1_1.csv.gz"),
    ("nai_shuffle_multirow_both_multimat_right_n_to_mn", "valid_n_to_mn_128_128_2_4_1_1.csv.gz"),
    ("nai_shuffle_multimat_right_work_distribution_n_to_mn", "valid_n_to_mn_10_10_2_4_1_1.csv.gz"),
    ("nai_shuffle_multirow_both_multimat_both_n_to_m", "valid_n_to_m_64_64_4_4_1_2.csv.gz"),
    ("nai_shuffle_multimat_both_work_distribution_n_to_m", "valid_n_to_m_10_10_4_4_1_1.csv.gz"),
    ("fft_orig_one_to_one", "valid_one_to_one_128_128_1_1_1_2.csv.gz"),
    ("fft_reduced_transfer_one_to_many", "valid_one_to_many_64_64_1_2_1_1.csv.gz"),
    ("fft_orig_n_to_mn", "valid_n_to_mn_128_128_2_4_1_1.csv.gz"),
    ("fft_better_n_to_m", "valid_n_to_m_64_64_4_2_1_1.csv.gz"),
    ("tc_bf16x3_one_to_one", "valid_one_to_one_64_64_1_1_1_2.csv.gz"),
    ("tc_bf16x3_n_to_mn", "valid_n_to_mn_128_128_2_4_1_1.csv.gz"),
    ("tc_bf16x3_n_to_m", "valid_n_to_m_64_64_4_4_1_2.csv.gz"),
    ("tc_tf32x3_n_to_mn", "valid_n_to_mn_128_128_2_4_1_1.csv.gz"),
]


def gunzip(tmp_path, path):
    import gzip
    dst = tmp_path / os.path.basename(path)[:-3]
    dst.write_bytes(gzip.open(path).read())
    return str(dst)


def cross(*args):
    return subprocess.run([CROSS, *args], capture_output=True, text=True)


@pytest.mark.parametrize("alg,name", CASES, ids=[c[0] for c in CASES])
def test_algorithm_against_golden(tmp_path, alg, name):
    mode, lp, rp, vp = golden_paths(name)
    assert alg.endswith(mode)
    lp, rp, vp = gunzip(tmp_path, lp), gunzip(tmp_path, rp), gunzip(tmp_path, vp)
    out = tmp_path / "out.csv"
    args = ["run", "-p", "-v", vp, "-o", str(out), alg, lp, rp]
    if alg.startswith("fft"):
        args.insert(1, "-n")
    r = cross(*args)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines()[0] == "Max,Mean,Stddev"
    res = oracle.read_csv(str(out))
    valid = oracle.read_csv(vp)
    assert res.shape == valid.shape
    assert rel_to_max(res, valid) <= 1e-5


def test_fft_raw_output_is_the_reference_layout(tmp_path):
    """Without -n the fft_* algorithms store the unnormalised 2H x 2W circular
    result, as the reference does (src/fft_alg.hpp:13-20)."""
    mode, lp, rp, vp = golden_paths("valid_one_to_many_64_64_1_2_1_1.csv.gz")
    lp, rp, vp = gunzip(tmp_path, lp), gunzip(tmp_path, rp), gunzip(tmp_path, vp)
    out = tmp_path / "raw.csv"
    r = cross("run", "-p", "-o", str(out), "fft_orig_one_to_many", lp, rp)
    assert r.returncode == 0, r.stderr
    raw = oracle.read_csv(str(out))
    assert raw.shape == (2, 128, 128)
    assert rel_to_max(oracle.normalize_fft(raw), oracle.read_csv(vp)) <= 1e-5
    # the CLI's own validate -n agrees
    r = cross("validate", "-n", "-c", vp, str(out))
    assert r.returncode == 0 and float(r.stdout.splitlines()[0].split(",")[0]) < 1e-2


@pytest.mark.parametrize("alg", ["nai_shuffle_one_to_one", "fft_orig_one_to_one"])
def test_double_precision(tmp_path, alg):
    name = "valid_one_to_one_10_10_1_1_1_2.csv.gz"
    assert name in FP64_EXACT
    mode, lp, rp, vp = golden_paths(name)
    lp, rp, vp = gunzip(tmp_path, lp), gunzip(tmp_path, rp), gunzip(tmp_path, vp)
    out = tmp_path / "out.csv"
    r = cross("run", "-p", "-n", "-d", "double", "-o", str(out), alg, lp, rp)
    assert r.returncode == 0, r.stderr
    assert rel_to_max(oracle.read_csv(str(out)), oracle.read_csv(vp)) <= 1e-12


def test_algorithm_timing_csv(tmp_path):
    mode, lp, rp, vp = golden_paths("valid_one_to_many_10_10_1_2_1_1.csv.gz")
    lp, rp = gunzip(tmp_path, lp), gunzip(tmp_path, rp)
    t = tmp_path / "times.csv"
    r = cross("run", "-p", "-b", "Algorithm", "-m", "0.01", "-t", str(t), "nai_shuffle_multimat_right_one_to_many",
              lp, rp)
    assert r.returncode == 0, r.stderr
    rows = t.read_text().strip().splitlines()
    assert rows[0] == "Kernel,Kernel_iterations,warps_per_thread_block,right_matrices_per_thread"
    ns, iters, w, m = rows[1].split(",")
    assert int(ns) > 0 and int(iters) >= 1 and (w, m) == ("8", "2")
    t2 = tmp_path / "fft.csv"
    r = cross("run", "-p", "-b", "Algorithm", "-m", "0.01", "-t", str(t2), "fft_orig_one_to_many", lp, rp)
    assert r.returncode == 0, r.stderr
    assert t2.read_text().splitlines()[0].startswith("Forward FFT,Forward FFT_iterations,Hadamard,")
    t3 = tmp_path / "compute.csv"
    r = cross("run", "-p", "-b", "Compute", "-m", "0.01", "-t", str(t3), "tc_bf16x3_one_to_many", lp, rp)
    assert r.returncode == 0, r.stderr
    assert t3.read_text().splitlines()[0] == "Computation,Computation_iterations"
