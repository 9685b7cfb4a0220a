"""Measure the timing dataset the method selector is trained on.

4096 seeded workloads: mode uniform over the four modes, square left and
right sides drawn log-uniformly from [16, 2048], batch (number of outputs)
log-uniform in [1, 256] (one_to_one: 1; one_to_many: M = batch; n_to_mn:
2 left, 2*ceil(batch/2) right; n_to_m: 2 left, ceil(batch/2) right), values
U[0,1).  Plus the 2048x2048 one_to_many batch of 16 right matrices.

Every candidate method (direct, fft, tc_bf16x3) is timed with CUDA events on
this GPU: one warm-up call, then the median of 3 calls (a single call when a
call takes more than 0.2 s).  Large batches are measured on a reduced batch
(outputs capped at 1 GiB and 2e12 algorithmic flops per call) and scaled
linearly to the full batch (every method's work is linear in the batch).
Methods that cannot run a workload (the split-BF16 path needs output width
<= 512 and right width <= 256) get time = inf.

Usage: python collect.py OUT.npz [--n 4096] [--seed 5]
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import xcorr  # noqa: E402

MODES = ["one_to_one", "one_to_many", "n_to_mn", "n_to_m"]
METHODS = ["direct", "fft", "tc_bf16x3"]


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


def counts(mode, batch):
    if mode == "one_to_one":
        return 1, 1
    if mode == "one_to_many":
        return 1, batch
    if mode == "n_to_mn":
        return 2, 2 * math.ceil(batch / 2)
    return 2, math.ceil(batch / 2)


def features(mode, sl, sr, batch):
    n_l, n_r = counts(mode, batch)
    n_out = xcorr.output_count(mode, n_l, n_r)
    return n_l, n_r, n_out


def time_call(fn, torch, long_s=0.2):
    fn()  # warm-up (plans, caches)
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) / 1000.0)
        if ts[-1] > long_s:
            break
    return float(np.median(ts))


def measure(mode, sl, sr, batch, torch, rng):
    n_l, n_r, n_out = features(mode, sl, sr, batch)
    S = (sl + sr - 1) ** 2
    flops_per_out = 2.0 * sl * sl * sr * sr
    cap = max(1, min(n_out, int(2 ** 30 / (4 * S)), int(2e12 / flops_per_out)))
    # reduced batch with the same mode structure
    if n_out > cap:
        m_l, m_r = counts(mode, cap)
        m_out = xcorr.output_count(mode, m_l, m_r)
    else:
        m_l, m_r, m_out = n_l, n_r, n_out
    scale = n_out / m_out
    left = torch.rand((m_l, sl, sl), device="cuda")
    right = torch.rand((m_r, sr, sr), device="cuda")
    out = torch.empty((m_out, sl + sr - 1, sl + sr - 1), device="cuda")
    res = []
    for method in METHODS:
        ws_b = xcorr.workspace_size(mode, "f32", method, (sl, sl), m_l, (sr, sr), m_r)
        ws = torch.empty(max(1, ws_b), dtype=torch.uint8, device="cuda") if ws_b else None
        try:
            t = time_call(lambda: xcorr.correlate(mode, left, right, method=method, out=out, workspace=ws), torch)
            res.append(t * scale)
        except xcorr.XcError:
            res.append(math.inf)
        del ws
    xcorr.lib().xc_release_thread_cache()
    del left, right, out
    return res, m_out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args()
    import torch

    wl = workloads(args.n, args.seed)
    rng = np.random.default_rng(args.seed + 1)
    times = np.full((len(wl), len(METHODS)), np.inf)
    measured_outputs = np.zeros(len(wl), dtype=np.int64)
    t0 = time.time()
    for i, (mode, sl, sr, b) in enumerate(wl):
        times[i], measured_outputs[i] = measure(mode, sl, sr, b, torch, rng)
        if i % 256 == 0:
            print(f"{i}/{len(wl)} {time.time() - t0:.0f}s", flush=True)
    np.savez_compressed(args.out, modes=np.array([w[0] for w in wl]), sides_left=np.array([w[1] for w in wl]),
                        sides_right=np.array([w[2] for w in wl]), batch=np.array([w[3] for w in wl]),
                        times=times, measured_outputs=measured_outputs, methods=np.array(METHODS),
                        gpu=np.array(torch.cuda.get_device_name(0)))
    print("done", time.time() - t0, "s")


if __name__ == "__main__":
    main()
