"""The banded schedule of the split tensor-core path, on the CPU.

When `xc_correlate_host` copies the output out in row bands while the kernel
runs, the host plans the bands and cuts each band's left rows into pieces that
it deals out to the CTAs (`csrc/tc_schedule.h`).  The kernel trusts that plan:
every tile's rows must be covered exactly once, pieces must stay within the
item size, each CTA must walk the bands in order, and the per-band piece counts
are what the host's copies wait for.  This compiles `band_schedule_check.cpp`
(which includes the header the CUDA source uses) with the host C++ compiler and
checks those invariants over a range of shapes, plus the balance that motivates
the plan.  No GPU needed."""
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
    exe = str(tmp_path_factory.mktemp("sched") / "band_schedule_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I" + CSRC, os.path.join(HERE, "band_schedule_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def run(exe, cases):
    text = "\n".join(" ".join(str(v) for v in c) for c in cases) + "\n"
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split("\n")
    return [line.split() for line in out if line]


def dy_of(k):
    """Row shifts per tile for k partners (partners per group: the next power of two, at most 128)."""
    p = 1
    while p < 128 and p < k:
        p *= 2
    return 128 // p


def cases():
    out = []
    # (Hl, Hr, partners, left matrices, shift halves, chunk_rows, bands, CTAs)
    shapes = [
        (256, 256, 64, 1, 2, 32, 8, 152),   # 1 x 64 right 256x256 (the bench workload)
        (256, 256, 64, 1, 2, 32, 2, 152),
        (256, 256, 64, 1, 2, 32, 4, 148),
        (200, 193, 1, 1, 2, 32, 8, 152),    # one_to_one 200x200 / 193x205
        (96, 89, 9, 1, 1, 16, 3, 152),      # small one_to_many
        (80, 73, 3, 2, 1, 8, 4, 152),       # n_to_mn 2 + 6
        (64, 57, 4, 3, 1, 4, 2, 12),        # n_to_m 3 x 4, few CTAs
        (512, 128, 32, 2, 2, 32, 8, 152),   # tall left
        (17, 300, 5, 1, 1, 4, 8, 152),      # short left, tall right
        (1, 1, 1, 1, 1, 4, 8, 152),         # one row each: a single tile
        (300, 300, 256, 1, 2, 32, 8, 152),  # 256 partners: one row shift per tile
        (40, 40, 2, 5, 2, 32, 5, 7),
    ]
    for hl, hr, k, nl, nh, cr, want, g in shapes:
        dy = dy_of(k)
        per_rank = nl * ((k + (128 // dy) - 1) // (128 // dy))
        out.append((hl, hr, dy, hl + hr - 1, per_rank, nh, cr, want, g, 16, 16 if nh == 2 else 0))
        # the kernel's own form: one item per tile key covers every shift
        out.append((hl, hr, dy, hl + hr - 1, per_rank, 1, cr, want, g, 34, 34))
    return out


def test_band_schedule_invariants(checker):
    cs = cases()
    res = run(checker, cs)
    assert len(res) == len(cs)
    for c, r in zip(cs, res):
        assert r[0] == "ok", f"case {c}: {' '.join(r)}"


def test_band_schedule_balance_at_the_bench_shape(checker):
    """1 x 64 right 256x256 in eight bands on 152 CTAs (64 partners x 2 row
    shifts per item, one item per tile key): the busiest CTA's modelled work
    within 3% of the mean.  (Cutting the bands into pieces of a quarter chunk
    would bring the ratio under 1% but raise the busiest CTA's work by 7%,
    every piece adding a drain.)"""
    (r,) = run(checker, [(256, 256, 2, 511, 1, 1, 32, 8, 152, 34, 34)])
    assert r[0] == "ok"
    max_load, mean = float(r[3]), float(r[4])
    assert max_load / mean <= 1.03, (max_load, mean)
