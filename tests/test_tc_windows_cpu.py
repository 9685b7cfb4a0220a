"""The MMA windows of the split tensor-core kernel, on the CPU.

Each K-step's MMA covers only the shifts whose overlap with the K-step's
right columns is non-empty, rounded out to 16 and placed in its shift half's
tensor-memory columns (`window_of` in `csrc/tc_schedule.h`, the function the
kernel's issuers call).  This compiles `tc_window_check.cpp` against that
header with the host C++ compiler and checks, over a range of shapes, that
every needed (shift, K-step) product is covered, that every window stays in
its half and its operand in the Toeplitz buffer, and that the windows issue
few MACs beyond the algorithmic ones.  No GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "cross-corr_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("win") / "tc_window_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I" + CSRC, os.path.join(HERE, "tc_window_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def run(exe, cases):
    text = "\n".join(" ".join(str(v) for v in c) for c in cases) + "\n"
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split("\n")
    return [line.split() for line in out if line]


SIDES_L = [1, 5, 17, 64, 100, 256, 300, 513, 700, 1000, 2048]
SIDES_R = [1, 3, 16, 40, 64, 255, 256, 257, 300, 520, 1024]


def test_windows_cover_every_needed_product_and_stay_in_bounds(checker):
    cases = [(wl, wr, tf) for tf in (0, 1) for wl in SIDES_L for wr in SIDES_R]
    for c, r in zip(cases, run(checker, cases)):
        assert r[0] == "ok", (c, r)


def test_windows_issue_few_macs_beyond_the_algorithmic_ones(checker):
    """At the bench shape (256 x 256) the windows issue 1.06x the algorithmic
    MACs (the 16-column rounding), against 1.5x for fixed 128-shift tiles
    that multiply the zero triangles where the diagonal crosses them."""
    (r,) = run(checker, [(256, 256, 0)])
    assert r[0] == "ok"
    ratio = int(r[1]) / int(r[2])
    assert 1.0 <= ratio <= 1.07, ratio
    for c, r in zip([(1000, 64, 0), (2048, 16, 0), (512, 512, 1)], run(checker, [(1000, 64, 0), (2048, 16, 0),
                                                                                (512, 512, 1)])):
        assert r[0] == "ok", c
        assert int(r[1]) / int(r[2]) <= 2.0, (c, r)
