"""Measure the timing dataset the algorithm selector is trained on.

4096 seeded workloads: mode uniform over the four modes, square left and
right sides drawn log-uniformly from [16, 2048], batch (number of outputs)
log-uniform in [1, 256] (one_to_one: 1; one_to_many: M = batch; n_to_mn:
2 left, 2*ceil(batch/2) right; n_to_m: 2 left, ceil(batch/2) right), values
U[0,1).  Plus the 2048x2048 one_to_many batch of 16 right matrices.

Every candidate algorithm (xc_algorithm: the plain kernel's three tiles, the
FFT path, split-BF16 with items of at most 32 or 64 rows, split-TF32) is
timed in the library with xc_time_algorithm: a warm-up call, then one call
between CUDA events, and when that call took under 20 ms a second
measurement of 3 calls, so no binding overhead is inside the timed region.
Large batches are measured on a reduced batch (outputs capped at 1 GiB,
algorithmic flops per call at 5e11) and scaled linearly to the full batch
(every candidate's work is linear in the batch).  Candidates that cannot
run a workload get time = inf.

Candidates are timed fastest-first (FFT, split paths, plain tiles).  A
candidate whose lower-bound time -- its algorithmic flops at the rate no
call of it can beat (the plain kernel: FP32 FMA peak, 152 SMs x 128 lanes x
2 flops x 2.07 GHz; the split paths: 3 or 6 products at the bf16 tensor
peak) -- is above 30 times the fastest time measured for the workload is
not run: the lower bound is recorded and `estimated` marks it.  Such a
candidate is never the fastest, and its bound still tells the network that
it is slow there.

The output is rewritten every 128 workloads (n_done says how many rows are
measured); --resume continues a partial file, --budget-s stops (after
saving) before a time limit.

Usage: python collect.py OUT.npz [--n 4096] [--seed 5] [--resume] [--budget-s S]
"""
from __future__ import annotations

import argparse
import ctypes
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import xcorr  # noqa: E402
from xcorr import selector  # noqa: E402

MODES = ["one_to_one", "one_to_many", "n_to_mn", "n_to_m"]


def workloads(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        mode = MODES[int(rng.integers(0, 4))]
        sl = int(round(2 ** rng.uniform(4, 11)))
        sr = int(round(2 ** rng.uniform(4, 11)))
        b = int(round(2 ** rng.uniform(0, 8)))
        out.append((mode, sl, sr, b))
    out.append(("one_to_many", 2048, 2048, 16))
    return out


# Rates no call of a candidate can beat (algorithmic flops per second): the
# plain kernel at the FP32 FMA peak, the split paths at the bf16 tensor peak
# over their 3 (BF16) or 6 (TF32: half the rate) products.
FMA_PEAK = 152 * 128 * 2 * 2.07e9
TENSOR_PEAK = 2.25e15
BOUND_RATE = {"direct": FMA_PEAK, "tc_bf16x3": TENSOR_PEAK / 3, "tc_tf32x3": TENSOR_PEAK / 6}
SKIP_FACTOR = 30.0
ORDER = ["fft", "tc_bf16x3:64", "tc_bf16x3:32", "tc_tf32x3", "direct:1", "direct:2", "direct:3"]


def time_algo(mode, dtype, algo, left, right, out, ws, wb, torch):
    """Seconds per call (xc_time_algorithm), or inf when unsupported."""
    L = xcorr.lib()
    n_l, sl, _ = left.shape
    n_r, sr, _ = right.shape
    ms = ctypes.c_double()
    st = torch.cuda.current_stream().cuda_stream
    args = (xcorr.MODES[mode], xcorr.DTYPES[dtype], algo, left.data_ptr(), xcorr.size2(sl, sl), n_l,
            right.data_ptr(), xcorr.size2(sr, sr), n_r, out.data_ptr(), ws, wb)
    if L.xc_time_algorithm(*args, 1, st, ctypes.byref(ms)) != 0:
        return math.inf
    if ms.value < 20.0 and L.xc_time_algorithm(*args, 3, st, ctypes.byref(ms)) != 0:
        return math.inf
    return ms.value / 1000.0


def measure(mode, sl, sr, batch, torch):
    """(times in seconds per full batch in ALGO_NAMES order, estimated flags,
    outputs measured)."""
    n_l, n_r = selector.counts(mode, batch)
    n_out = xcorr.output_count(mode, n_l, n_r)
    S = (sl + sr - 1) ** 2
    flops_per_out = 2.0 * sl * sl * sr * sr
    cap = max(1, min(n_out, int(2 ** 30 / (4 * S)), int(5e11 / flops_per_out)))
    # reduced batch with the same mode structure
    if n_out > cap:
        m_l, m_r = selector.counts(mode, cap)
        m_out = xcorr.output_count(mode, m_l, m_r)
    else:
        m_l, m_r, m_out = n_l, n_r, n_out
    scale = n_out / m_out
    left = torch.rand((m_l, sl, sl), device="cuda")
    right = torch.rand((m_r, sr, sr), device="cuda")
    out = torch.empty((m_out, sl + sr - 1, sl + sr - 1), device="cuda")
    res = {}
    est = {}
    best = math.inf
    for name in ORDER:
        algo = selector.algo_struct(name)
        base = name.partition(":")[0]
        est[name] = False
        try:
            wb = xcorr.workspace_size(mode, "f32", base, (sl, sl), m_l, (sr, sr), m_r)
        except xcorr.XcError:
            res[name] = math.inf
            continue
        bound = flops_per_out * m_out / BOUND_RATE[base] if base in BOUND_RATE else 0.0
        if bound > SKIP_FACTOR * best:
            res[name] = bound * scale
            est[name] = True
            continue
        ws = torch.empty(max(1, wb), dtype=torch.uint8, device="cuda")
        t = time_algo(mode, "f32", algo, left, right, out, ws.data_ptr(), wb, torch)
        del ws
        best = min(best, t)
        res[name] = t * scale
    xcorr.lib().xc_release_thread_cache()
    del left, right, out
    return [res[n] for n in selector.ALGO_NAMES], [est[n] for n in selector.ALGO_NAMES], m_out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--resume", action="store_true")
    ap.add_argument("--budget-s", type=float, default=0.0, help="save and stop after this many seconds (0: no limit)")
    args = ap.parse_args()
    import torch

    wl = workloads(args.n, args.seed)
    times = np.full((len(wl), len(selector.ALGO_NAMES)), np.inf)
    estimated = np.zeros((len(wl), len(selector.ALGO_NAMES)), dtype=bool)
    measured_outputs = np.zeros(len(wl), dtype=np.int64)
    start = 0
    if args.resume and os.path.exists(args.out):
        z = np.load(args.out)
        start = int(z["n_done"])
        times[:start] = z["times"][:start]
        estimated[:start] = z["estimated"][:start]
        measured_outputs[:start] = z["measured_outputs"][:start]
    t0 = time.time()

    def save(n_done):
        # rows past n_done are not measured yet (all inf, measured_outputs 0)
        np.savez_compressed(args.out, modes=np.array([w[0] for w in wl]), sides_left=np.array([w[1] for w in wl]),
                            sides_right=np.array([w[2] for w in wl]), batch=np.array([w[3] for w in wl]),
                            times=times, estimated=estimated, measured_outputs=measured_outputs,
                            algorithms=np.array(selector.ALGO_NAMES), gpu=np.array(torch.cuda.get_device_name(0)),
                            n_done=np.array(n_done))

    for i, (mode, sl, sr, b) in enumerate(wl):
        if i < start:
            continue
        times[i], estimated[i], measured_outputs[i] = measure(mode, sl, sr, b, torch)
        if i % 128 == 127:
            print(f"{i + 1}/{len(wl)} {time.time() - t0:.0f}s", flush=True)
            save(i + 1)
            if args.budget_s and time.time() - t0 > args.budget_s:
                print("budget reached; continue with --resume", flush=True)
                return
    save(len(wl))
    print("done", time.time() - t0, "s")


if __name__ == "__main__":
    main()
