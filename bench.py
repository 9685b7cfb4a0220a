"""Benchmark: correlations/s at <= 1e-5 relative error vs FP64.

Workload (one GPU): one_to_many, FP32, one left 256x256 and 64 right 256x256
matrices, values i.i.d. uniform [0,1) from a fixed seed; 64 full outputs of
511x511.  Synthetic data with the configuration's shapes and distribution.

A step is one batched correlation of the whole workload.  `value` counts the
correlations (output matrices) completed per second with inputs already in
HBM, timed with CUDA events on the launching stream; L2 is flushed (a 256 MiB
write) before every timed step, outside the timed region.  `e2e` is the same
metric through the C ABI's host-buffer entry points with pinned host buffers:
every step's host->device copy, correlation and device->host copy inside the
timed region, the steps issued as a stream of calls with two in flight
(xc_correlate_host_async), so one call's copies overlap its neighbours'
kernels; the one-call-at-a-time figure (xc_correlate_host) is reported beside
it.  Every reported output is checked against an FP64
reference before the number is printed (all 64 outputs against an FP64 FFT
on the GPU, two of them also against the CPU oracle).

`--impl reference` times the reference's CPU algorithm (cpu_cross_corr_*,
restated in C as oracle/xcorr_oracle.c because the reference's own CPU code
needs Boost) on the host cores, on a bounded sample of pairs per step.

Launch: python bench.py [--gpus N --steps K --warmup W]; for N>1 under
torchrun each rank runs the same per-GPU workload (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cross-corr_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

WORKLOAD = {"workload": "one_to_many fp32 256x256 x 64 right", "mode": "one_to_many", "left": [1, 256, 256],
            "right": [64, 256, 256], "distribution": "uniform[0,1)", "seed": 2}
METRIC = "correlations/s at <=1e-5 rel err vs FP64"
GATE = 1e-5


def make_inputs():
    rng = np.random.default_rng(WORKLOAD["seed"])
    left = rng.random(WORKLOAD["left"]).astype(np.float32)
    right = rng.random(WORKLOAD["right"]).astype(np.float32)
    return left, right


def algorithmic_flops(left_shape, right_shape, pairs):
    return 2.0 * left_shape[-2] * left_shape[-1] * right_shape[-2] * right_shape[-1] * pairs


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, \
            "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms by one background
    nvidia-smi process that runs for the duration of the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.splitlines():
            cols = [c.strip() for c in line.split(",")]
            if len(cols) >= 9:
                self.rows.append(cols)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in self.rows) if v is not None]
        mx = [v for v in (num(r[2]) for r in self.rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_reference_rate(left, right, pairs: int, threads: int):
    """Reference CPU algorithm (T=float, oracle/xcorr_oracle.c restatement of
    cpu_cross_corr_one_to_many) on `pairs` right matrices; returns pairs/s."""
    from oracle import oracle

    t0 = time.perf_counter()
    oracle.run_mode("one_to_many", left, right[:pairs], dtype="f32", threads=threads)
    dt = time.perf_counter() - t0
    return pairs / dt, dt


def scipy_reference_rate(left, right, pairs: int = 1):
    """The reference's Python implementation computes each pair with
    scipy.signal.correlate2d(L, R, 'full') (existing/python/crosscorr.py);
    that call, timed on one host thread over `pairs` pairs of the workload.
    None when SciPy is not installed."""
    try:
        from scipy import signal
    except ImportError:
        return None
    L = left[0].astype(np.float32)
    t0 = time.perf_counter()
    for k in range(pairs):
        signal.correlate2d(L, right[k].astype(np.float32), mode="full")
    dt = time.perf_counter() - t0
    return {"value": pairs / dt, "unit": "correlations/s", "cores": 1,
            "sample": f"{pairs} of 64 pairs ({dt:.1f} s), scipy.signal.correlate2d(L, R, 'full'), float32"}


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    left, right = make_inputs()
    threads = os.cpu_count() or 1
    sample = 16  # pairs per step: ~6.9e10 MACs, several seconds on 16 cores
    for _ in range(args.warmup):
        cpu_reference_rate(left, right, 1, threads)
    t_total, pairs_total = 0.0, 0
    for _ in range(args.steps):
        _, dt = cpu_reference_rate(left, right, sample, threads)
        t_total += dt
        pairs_total += sample
    value = pairs_total / t_total
    line = {
        "metric": METRIC, "value": value, "unit": "correlations/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": dict(WORKLOAD, parallelism="host threads"),
        "cpu_baseline": {"value": value, "unit": "correlations/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of 64 pairs per step (cpu_cross_corr_one_to_many restated in C, "
                                   f"T=float, {threads} threads)"},
        "e2e": {"value": value, "unit": "correlations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_gate(out_dev, left, right, torch, xcorr):
    """All outputs vs an FP64 FFT on the GPU; two outputs vs the CPU oracle."""
    from oracle import oracle

    l64 = torch.from_numpy(left).double().cuda()
    r64 = torch.from_numpy(right).double().cuda()
    ref = xcorr.correlate("one_to_many", l64, r64, method="fft")
    torch.cuda.synchronize()
    o = out_dev.double()
    err = ((o - ref).abs().amax(dim=(1, 2)) / ref.abs().amax(dim=(1, 2))).max().item()
    o_cpu = out_dev[:2].cpu().numpy()
    ref_cpu = oracle.run_mode("one_to_many", left, right[:2], dtype="f32acc64", threads=os.cpu_count() or 1)
    err_oracle = max(oracle.max_rel_to_max(o_cpu[k], ref_cpu[k]) for k in range(2))
    del l64, r64, ref
    return max(err, err_oracle), err, err_oracle


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    import xcorr

    torch.cuda.set_device(local_rank)
    xcorr.check(xcorr.lib().xc_device_check(local_rank))
    left, right = make_inputs()
    pairs = right.shape[0]
    dl = torch.from_numpy(left).cuda()
    dr = torch.from_numpy(right).cuda()
    method = args.method
    out = torch.empty((pairs, 511, 511), device="cuda", dtype=torch.float32)
    ws_bytes = xcorr.workspace_size("one_to_many", "f32", method, (256, 256), 1, (256, 256), pairs)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def make_step(m, o, w, wb):
        def step():
            xcorr.correlate("one_to_many", dl, dr, method=m, out=o, workspace=w if wb else None)
        return step

    step = make_step(method, out, ws, ws_bytes)

    def timed(fn, steps):
        """Per-step CUDA-event times (ms), L2 flushed before each step."""
        ts = []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return ts

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    gate, gate_fft, gate_oracle = accuracy_gate(out, left, right, torch, xcorr)
    if gate > GATE:
        raise SystemExit(f"accuracy gate failed: {gate:.3e} > {GATE}")

    # ---- device-resident timing: per-step CUDA events, L2 flushed between steps
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk, xcorr.kernel_timing() as kt:
        times = timed(step, args.steps)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = sum(times) / len(times)

    # ---- the plain FP32 kernel on the same inputs (the comparison the metric names)
    plain = None
    if method != "direct":
        out_p = torch.empty_like(out)
        step_p = make_step("direct", out_p, None, 0)
        for _ in range(args.warmup):
            step_p()
        torch.cuda.synchronize()
        gate_p, _, _ = accuracy_gate(out_p, left, right, torch, xcorr)
        ts_p = timed(step_p, args.steps)
        ms_p = sum(ts_p) / len(ts_p)
        plain = {"value": pairs / (ms_p / 1000.0), "ms_per_step": ms_p, "max_rel_err_vs_fp64": gate_p,
                 "method": "direct (plain FP32 FMA kernel)", "speedup_of_headline": ms_p / ms}
        del out_p
    # ---- the split-TF32 arm on the same inputs (more accurate, half the tensor rate)
    tf32 = None
    if method == "tc_bf16x3":
        out_t = torch.empty_like(out)
        wb_t = xcorr.workspace_size("one_to_many", "f32", "tc_tf32x3", (256, 256), 1, (256, 256), pairs)
        ws_t = torch.empty(max(wb_t, 1), dtype=torch.uint8, device="cuda")
        step_t = make_step("tc_tf32x3", out_t, ws_t, wb_t)
        for _ in range(args.warmup):
            step_t()
        torch.cuda.synchronize()
        gate_t, _, _ = accuracy_gate(out_t, left, right, torch, xcorr)
        ts_t = timed(step_t, args.steps)
        ms_t = sum(ts_t) / len(ts_t)
        tf32 = {"value": pairs / (ms_t / 1000.0), "ms_per_step": ms_t, "max_rel_err_vs_fp64": gate_t,
                "method": "tc_tf32x3 (split-TF32 tensor cores)"}
        del out_t, ws_t
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = t.item()
    value = pairs * world / (ms_max / 1000.0)

    # ---- end to end through the C ABI host-buffer call (pinned host memory)
    hl = torch.from_numpy(left).pin_memory()
    hr = torch.from_numpy(right).pin_memory()
    ho = torch.empty((pairs, 511, 511), dtype=torch.float32).pin_memory()
    L = xcorr.lib()

    def e2e_step():
        xcorr.check(L.xc_correlate_host(xcorr.MODES["one_to_many"], 0, xcorr.METHODS[method], hl.data_ptr(),
                                        xcorr.size2(256, 256), 1, hr.data_ptr(), xcorr.size2(256, 256), pairs,
                                        ho.data_ptr(), stream.cuda_stream))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()  # synchronises the stream before returning
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_times) / len(e2e_times)
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = t.item()
    e2e_err = float(np.abs(ho.numpy()[:2].astype(np.float64) - out[:2].cpu().numpy()).max())
    # the host-buffer call may cut the work differently (output bands): the
    # same accuracy gate as the device-resident output
    gate_e2e, _, _ = accuracy_gate(ho.cuda(), left, right, torch, xcorr)
    if gate_e2e > GATE:
        raise SystemExit(f"accuracy gate failed on the host-buffer output: {gate_e2e:.3e} > {GATE}")

    # ---- the same problem as a stream of host-buffer calls: two in flight
    # (xc_correlate_host_async), so one call's copies run under the other's
    # kernel; each call still copies its inputs in and its output out.  The
    # outputs alternate between two pinned buffers, as a caller consuming
    # results while the next call runs would.
    hln, hrn = hl.numpy(), hr.numpy()
    hos = [ho.numpy(), torch.empty((pairs, 511, 511), dtype=torch.float32).pin_memory().numpy()]

    def e2e_stream(n):
        pending = []
        t0 = time.perf_counter()
        for i in range(n):
            if len(pending) == 2:  # the output buffer about to be reused is read first
                xcorr.host_wait(pending.pop(0))
            pending.append(xcorr.correlate_host_async("one_to_many", hln, hrn, hos[i % 2], method=method,
                                                      stream=stream.cuda_stream))
        for t in pending:
            xcorr.host_wait(t)
        return time.perf_counter() - t0

    e2e_stream(max(3, args.warmup))
    for h in hos:
        h.fill(np.nan)
    torch.cuda.synchronize()
    with xcorr.kernel_timing() as kt_stream:
        stream_s = e2e_stream(args.steps) / args.steps
    if world > 1:
        t = torch.tensor([stream_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        stream_s = t.item()
    gate_stream = max(accuracy_gate(torch.from_numpy(h).cuda(), left, right, torch, xcorr)[0] for h in hos)
    if gate_stream > GATE:
        raise SystemExit(f"accuracy gate failed on the pipelined host-buffer output: {gate_stream:.3e} > {GATE}")

    peaks, peak_src = measured_peaks()
    flops = algorithmic_flops(left.shape, right.shape, pairs)
    kernel_ms = kt.total_ms / kt.launches if kt.launches else None
    achieved = flops / ((kernel_ms if kernel_ms else ms) / 1000.0) / 1e12
    if method == "tc_bf16x3":
        bound, peak, unit = "tensor", float(peaks.get("bf16_tflops", 1900.0)), "TFLOP/s"
        peak_note = f"{peak_src} cuBLAS bf16 burst; algorithmic FP32 flops (3 bf16 products each)"
    elif method == "tc_tf32x3":
        bound, peak, unit = "tensor", float(peaks.get("bf16_tflops", 1900.0)) / 2, "TFLOP/s"
        peak_note = (f"half the {peak_src} cuBLAS bf16 burst (a TF32 MMA does half the K of a BF16 one in the "
                     "same time); algorithmic FP32 flops (3 tf32 products each)")
    else:
        mhz = float(peaks.get("sm_max_mhz", 2070.0))
        bound, peak, unit = "fp32", 152 * 128 * 2 * mhz * 1e6 / 1e12, "TFLOP/s"
        peak_note = "nominal FP32 FMA peak (152 SMs x 128 lanes x 2 x max SM clock); no measured SIMT peak exists"
    clocks = clk.summary()
    kernel_name = "tc_kernel" if method.startswith("tc_") else "direct_kernel"
    line = {
        "metric": METRIC, "value": value, "unit": "correlations/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(WORKLOAD, method=method, l2="flushed (256 MiB write) before every timed step",
                       parallelism=f"replica per GPU x{world}"),
        "accuracy": {"max_rel_err_vs_fp64": gate, "vs_gpu_fp64_fft_all_outputs": gate_fft,
                     "vs_cpu_oracle_2_outputs": gate_oracle, "gate": GATE},
        "e2e": {"value": pairs * world / stream_s, "unit": "correlations/s",
                "h2d_bytes_per_step": int(left.nbytes + right.nbytes), "d2h_bytes_per_step": int(ho.numel() * 4),
                "api": "xc_correlate_host_async + xc_host_wait (pinned host buffers, two calls in flight: each "
                       "call's copy-in and copy-out overlap the neighbouring calls' kernels)",
                "ms_per_step": stream_s * 1000.0, "max_rel_err_vs_fp64": gate_stream,
                "kernel_ms": kt_stream.total_ms / kt_stream.launches if kt_stream.launches else None,
                "l2": "inputs copied in from host memory every step; the two slots' buffers and the workspace "
                      "(about 220 MB) exceed L2",
                "synchronous": {"value": pairs * world / e2e_s, "ms_per_step": e2e_s * 1000.0,
                                "api": "xc_correlate_host (one call at a time, L2 flushed before each)",
                                "max_abs_diff_vs_device_run": e2e_err, "max_rel_err_vs_fp64": gate_e2e}},
        "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak,
                     # a split product costs 3 tensor-core products: the split path's ceiling is peak / 3
                     "split_products": 3 if method.startswith("tc_") else None,
                     "frac_of_split_ceiling": (achieved * 3 / peak) if method.startswith("tc_") else None,
                     "traffic": profiled_traffic(kernel_name), "kernel": kernel_name,
                     "algorithmic_flops_per_launch": flops, "peak_source": peak_note,
                     "kernel_ms": kernel_ms, "kernel_launches_timed": kt.launches,
                     "kernel_share_of_step": (kernel_ms / ms) if kernel_ms else None,
                     "duration": "CUDA events around each launch of the kernel on its stream, inside the timed "
                                 "region (xc_kernel_timing)",
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch, ncu capture "
                                       f"summarised in profiles/{kernel_name}_one_to_many_256x64.md"},
        "clocks": clocks,
        "gpu_launches": gpu_launches(method, args.steps),
    }
    if method == "fft":
        # the step is two cuFFT transforms around four glue kernels: the
        # transforms are the library's, timed but not modelled; the glue
        # kernels' HBM fractions come from their own captures
        line["roofline"] = {"bound": "hbm", "achieved": None, "peak": float(peaks.get("hbm_gbs", 6800.0)),
                            "unit": "GB/s", "frac": None, "traffic": None, "kernel": "fft step",
                            "note": "cuFFT transforms plus pad, conj-multiply and normalise kernels; the glue "
                                    "kernels' achieved GB/s against this peak are in "
                                    "profiles/fft_glue_one_to_many_256x64.md"}
    if plain is not None:
        line["plain_fp32"] = plain
    if tf32 is not None:
        line["tf32x3"] = tf32
    if rank == 0 and not args.no_ragged:
        line["ragged_n_to_m"] = ragged_study(torch, xcorr)
    if rank == 0 and not args.no_configs:
        line["configs"] = config_studies(torch, xcorr)
        line["large_fft"] = large_fft_study(torch, xcorr)
        line["templates"] = template_study(torch, xcorr)
    if rank == 0 and not args.no_csv:
        line["csv_io"] = csv_study(xcorr)
    if rank == 0 and not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_study(torch, xcorr, line)
    if rank == 0 and not args.no_cpu_baseline:
        rate, dt = cpu_reference_rate(left, right, 16, os.cpu_count() or 1)
        # the reference's cpu_* are single-threaded by construction: one core too
        rate1, dt1 = cpu_reference_rate(left, right, 1, 1)
        line["cpu_baseline"] = {"value": rate, "unit": "correlations/s", "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": f"16 of 64 pairs ({dt:.1f} s), cpu_cross_corr_one_to_many "
                                                          "restated in C, T=float",
                                "single_core": {"value": rate1, "cores": 1,
                                                "sample": f"1 of 64 pairs ({dt1:.1f} s), the same loop on one thread"}}
        scipy_rate = scipy_reference_rate(left, right)
        if scipy_rate is not None:
            line["cpu_baseline"]["scipy_correlate2d"] = scipy_rate
    if rank == 0:
        print(json.dumps(line), flush=True)


def csv_study(xcorr, loops=3):
    """CSV throughput of the `cross` CLI, the reference's on-disk format
    (`# rows,cols,count` header, one matrix row per line; src/matrix.hpp:94-185):
    the workload's inputs (1 + 64 matrices of 256x256, written by numpy with
    9 significant digits) are loaded and the 64 outputs of 511x511 stored by
    `cross run -b CommonSteps`, whose Load and Store columns time exactly
    those steps (nanoseconds per loop, `loops` loops; the median is kept)."""
    import csv
    import tempfile

    left, right = make_inputs()
    with tempfile.TemporaryDirectory() as d:
        paths = {}
        for name, a in (("left", left), ("right", right)):
            paths[name] = os.path.join(d, f"{name}.csv")
            with open(paths[name], "w") as f:
                f.write(f"# {a.shape[1]},{a.shape[2]},{a.shape[0]}\n")
                np.savetxt(f, a.reshape(-1, a.shape[2]), delimiter=",", fmt="%.9g")
        times, out = os.path.join(d, "times.csv"), os.path.join(d, "out.csv")
        r = subprocess.run([xcorr.CLI_PATH, "run", "-b", "CommonSteps", "-l", str(loops), "-m", "0", "-t", times,
                            "-o", out, "nai_shuffle_multimat_right_one_to_many", paths["left"], paths["right"]],
                           capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            return {"error": (r.stderr or r.stdout).strip()[-300:]}
        with open(times) as f:
            rows = list(csv.DictReader(f))
        load_ms = statistics.median(float(row["Load"]) for row in rows) / 1e6
        store_ms = statistics.median(float(row["Store"]) for row in rows) / 1e6
        in_bytes = os.path.getsize(paths["left"]) + os.path.getsize(paths["right"])
        out_bytes = os.path.getsize(os.path.join(d, "out_0.csv"))
    return {"command": "cross run -b CommonSteps nai_shuffle_multimat_right_one_to_many", "loops": loops,
            "input_mb": in_bytes / 1e6, "output_mb": out_bytes / 1e6, "load_ms": load_ms, "store_ms": store_ms,
            "load_mb_per_s": in_bytes / 1e3 / load_ms, "store_mb_per_s": out_bytes / 1e3 / store_ms,
            "values_per_s_load": (left.size + right.size) / (load_ms / 1e3),
            "values_per_s_store": 64 * 511 * 511 / (store_ms / 1e3), "host_threads": os.cpu_count()}


def sampled_fp64(left, right, outs, ref_scale, rng, n_shifts):
    """Max |out - exact| / scale over `n_shifts` shifts per output, each
    summed in FP64 on the CPU (numpy) straight from the definition
    out[sy + Hr-1][sx + Wr-1] = sum L[y+sy][x+sx] R[y][x]; every output also
    gets its centre shift (the longest sum).  left (Hl, Wl), right (m, Hr,
    Wr), outs (m, Sy, Sx) for one_to_many; scale[k] = max|exact| of output k."""
    hl, wl = left.shape
    _, hr, wr = right.shape
    L = left.astype(np.float64)
    worst = 0.0
    for k in range(right.shape[0]):
        R = right[k].astype(np.float64)
        sys_ = np.concatenate([[hr - 1], rng.integers(0, hl + hr - 1, n_shifts - 1)])
        sxs = np.concatenate([[wr - 1], rng.integers(0, wl + wr - 1, n_shifts - 1)])
        for oy, ox in zip(sys_, sxs):
            dy, dx = int(oy) - (hr - 1), int(ox) - (wr - 1)
            y0, y1 = max(0, -dy), min(hr, hl - dy)
            x0, x1 = max(0, -dx), min(wr, wl - dx)
            exact = float(np.sum(L[y0 + dy:y1 + dy, x0 + dx:x1 + dx] * R[y0:y1, x0:x1]))
            worst = max(worst, abs(float(outs[k][oy, ox]) - exact) / ref_scale[k])
    return worst


def template_study(torch, xcorr, reps=5):
    """Small templates on large lefts (one_to_many, U[0,1), seed 6): 16 right
    matrices of 16x16, 32x32 or 64x64 on a left of 256x256 to 2048x2048, the
    regime where the FFT path transforms the whole padded left for a few
    small products.  Every method's time and its error against the library's
    FP64 FFT; the fastest at <= 1e-5 is named."""
    out = []
    for side in (256, 512, 1024, 2048):
        for t in (16, 32, 64):
            rng = np.random.default_rng(6)
            left = torch.from_numpy(rng.random((1, side, side)).astype(np.float32)).cuda()
            right = torch.from_numpy(rng.random((16, t, t)).astype(np.float32)).cuda()
            ref = xcorr.correlate("one_to_many", left.double(), right.double(), method="fft")
            scale = ref.abs().amax(dim=(1, 2))
            row = {"left": side, "template": t, "rights": 16}
            best = None
            for method in ("direct", "fft", "tc_bf16x3"):
                ws_bytes = xcorr.workspace_size("one_to_many", "f32", method, (side, side), 1, (t, t), 16)
                ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
                o = xcorr.correlate("one_to_many", left, right, method=method, workspace=ws if ws_bytes else None)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    xcorr.correlate("one_to_many", left, right, method=method, out=o, workspace=ws if ws_bytes else None)
                e1.record()
                e1.synchronize()
                ms = e0.elapsed_time(e1) / reps
                err = float(((o.double() - ref).abs().amax(dim=(1, 2)) / scale).max())
                row[method] = {"ms": ms, "max_rel_err_vs_fp64": err}
                if err <= GATE and (best is None or ms < row[best]["ms"]):
                    best = method
                del o, ws
            row["fastest_within_gate"] = best
            out.append(row)
            del left, right, ref
    torch.cuda.empty_cache()
    return out


def large_fft_study(torch, xcorr, reps=5):
    """one_to_many FP32 FFT, left 2048x2048 and 16 right 2048x2048 (U[0,1),
    seed 5): 16 outputs of 4095x4095 from 4096x4096 transforms, where the
    normalisation scales in FP64.  Error against the library's FP64 FFT
    (all 16 outputs, full) and against FP64 sums on the CPU at 64 sampled
    shifts per output (centre shift included)."""
    rng = np.random.default_rng(5)
    left = rng.random((1, 2048, 2048)).astype(np.float32)
    right = rng.random((16, 2048, 2048)).astype(np.float32)
    dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    ws_bytes = xcorr.workspace_size("one_to_many", "f32", "fft", (2048, 2048), 1, (2048, 2048), 16)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    o = xcorr.correlate("one_to_many", dl, dr, method="fft", workspace=ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        xcorr.correlate("one_to_many", dl, dr, method="fft", out=o, workspace=ws)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del ws
    # the FP64 FFT of the same inputs, output by output (one right at a time
    # keeps the FP64 workspace near 1 GB)
    errs_fft, scales = [], []
    dl64 = dl.double()
    for k in range(16):
        ref = xcorr.correlate("one_to_many", dl64, dr[k:k + 1].double(), method="fft")[0]
        scale = float(ref.abs().max())
        errs_fft.append(float((o[k].double() - ref).abs().max()) / scale)
        scales.append(scale)
        del ref
    host = o.cpu().numpy()
    err_cpu = sampled_fp64(left[0], right, host, scales, np.random.default_rng(55), 64)
    del o, dl, dr, dl64
    torch.cuda.empty_cache()
    return {"config": "one_to_many 2048x2048 x 16 right U[0,1) seed 5", "dtype": "f32", "method": "fft",
            "transform": [4096, 4096], "outputs": 16, "output_shape": [4095, 4095],
            "correlations_per_s": 16 / (ms / 1000.0), "ms": ms,
            "max_rel_err_vs_gpu_fp64_fft_all_outputs": max(errs_fft),
            "max_rel_err_vs_cpu_fp64_64_sampled_shifts_per_output": err_cpu}


def ragged_study(torch, xcorr, reps=5):
    """Ragged n_to_m batch (512 pairs, every side drawn from U{16..512}, values
    U[-1,1), seed 4): the graph-captured plan with its autotuned variant (tile
    shape of the persistent plain kernel, and the pairs routed to the
    split-BF16 path) against the same plan with every pair on the plain
    kernel, and against one plain-kernel launch per pair, on one stream and
    round-robin over 8 streams (the reference's driver).  The CPU oracle
    checks the 24 smallest and the 8 largest pairs (about 270 GMAC, run in a
    background thread while the GPU timings run)."""
    import tempfile

    from oracle import oracle

    os.environ.setdefault("XC_AUTOTUNE_CACHE", os.path.join(tempfile.gettempdir(), "xcorr_bench_autotune.jsonl"))
    rng = np.random.default_rng(4)
    lefts, rights = [], []
    for _ in range(512):
        hl, wl, hr, wr = rng.integers(16, 513, size=4)
        lefts.append(rng.uniform(-1, 1, (hl, wl)).astype(np.float32))
        rights.append(rng.uniform(-1, 1, (hr, wr)).astype(np.float32))
    pairs = [(i, i) for i in range(512)]
    by_work = sorted(range(512), key=lambda i: lefts[i].size * rights[i].size)
    small, large = by_work[:24], by_work[-8:]
    checked = small + large
    refs = {}

    def run_oracle():
        res = oracle.run_pairs([lefts[i] for i in checked], [rights[i] for i in checked],
                               threads=os.cpu_count() or 1)
        refs.update(zip(checked, res))

    worker = threading.Thread(target=run_oracle)
    worker.start()
    plan = xcorr.RaggedPlan(lefts, rights, pairs)
    variant, tune_ms = plan.autotune()
    chosen = plan.describe()
    base = torch.zeros_like(plan.out)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    # the chosen variant's tile shape with every pair on the plain kernel
    plan.select(chosen["tile_shape"])
    ms_plain = timed(plan.execute)
    plain_outs = plan.outputs()
    plan.select(variant)
    ms_graph = timed(plan.execute)
    ms_pairs = timed(lambda: plan.per_pair(base))
    base8 = torch.zeros_like(plan.out)
    ms_streams = timed(lambda: plan.per_pair_streams(base8, 8))
    outs, outs_b = plan.outputs(), plan.outputs(base)
    diff = max(oracle.max_rel_to_max(a, b) for a, b in zip(outs, outs_b))
    diff8 = max(oracle.max_rel_to_max(a, b) for a, b in zip(outs, plan.outputs(base8)))
    worker.join()
    err = max(oracle.max_rel_to_max(outs[i], refs[i]) for i in small)
    err_large = max(oracle.max_rel_to_max(outs[i], refs[i]) for i in large)
    err_large_pp = max(oracle.max_rel_to_max(outs_b[i], refs[i]) for i in large)
    err_plain = max(oracle.max_rel_to_max(plain_outs[i], refs[i]) for i in checked)
    flops = sum(2.0 * l.size * r.size for l, r in zip(lefts, rights))
    plan.close()
    return {"pairs": 512, "sides": "U{16..512} each of Hl, Wl, Hr, Wr", "values": "U[-1,1)", "seed": 4,
            "persistent_graph_ms": ms_graph, "per_pair_launches_ms": ms_pairs, "speedup": ms_pairs / ms_graph,
            "per_pair_launches_8_streams_ms": ms_streams, "speedup_vs_8_streams": ms_streams / ms_graph,
            "autotuned_variant": chosen, "autotune_ms": tune_ms,
            "plain_kernel_only": {"ms": ms_plain, "tflops": flops / (ms_plain / 1000.0) / 1e12,
                                  "max_rel_err_vs_oracle_32_checked_pairs": err_plain,
                                  "speedup_of_chosen_variant": ms_plain / ms_graph},
            "correlations_per_s": 512 / (ms_graph / 1000.0), "tflops": flops / (ms_graph / 1000.0) / 1e12,
            "max_rel_err_vs_oracle_24_smallest_pairs": err,
            "max_rel_err_vs_oracle_8_largest_pairs": err_large,
            "largest_pairs_sides": [list(lefts[i].shape) + list(rights[i].shape) for i in large],
            "per_pair_launches_max_rel_err_vs_oracle_8_largest_pairs": err_large_pp,
            "max_rel_diff_graph_vs_per_pair": diff, "max_rel_diff_graph_vs_8_streams": diff8}


def profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` at this workload, read from its
    committed ncu summary (a line `traffic_bytes_per_launch: N`), or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_one_to_many_256x64.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def config_studies(torch, xcorr, reps=20):
    """The other fixed configurations, each method's rate and error vs FP64:
    one_to_one 128x128 (U[0,1), seed 1); 8 left + 32 right 64x64 N(0,1)
    (seed 3) as n_to_mn (32 outputs) and as n_to_m (256 outputs), in FP32 and
    FP64.  Inputs are small (L2-resident); each rate is the mean of `reps`
    back-to-back calls after a warm-up call."""
    from oracle import oracle

    cases = []
    rng = np.random.default_rng(1)
    a, b = rng.random((1, 128, 128)), rng.random((1, 128, 128))
    cases.append(("one_to_one 128x128 U[0,1) seed 1", "one_to_one", a, b))
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal((8, 64, 64)), rng.standard_normal((32, 64, 64))
    cases.append(("n_to_mn 8+32 x 64x64 N(0,1) seed 3", "n_to_mn", a, b))
    cases.append(("n_to_m 8+32 x 64x64 N(0,1) seed 3", "n_to_m", a, b))
    out = []
    threads = os.cpu_count() or 1
    for name, mode, a, b in cases:
        for dtype in ("f32", "f64"):
            np_t = np.float32 if dtype == "f32" else np.float64
            la, rb = a.astype(np_t), b.astype(np_t)
            ref = oracle.run_mode(mode, la, rb, dtype="f64" if dtype == "f64" else "f32acc64", threads=threads)
            dl, dr = torch.from_numpy(la).cuda(), torch.from_numpy(rb).cuda()
            row = {"config": name, "dtype": dtype, "outputs": int(ref.shape[0])}
            for method in ("direct", "fft", "tc_bf16x3", "tc_tf32x3"):
                if method.startswith("tc_") and dtype == "f64":
                    continue
                ws_bytes = xcorr.workspace_size(mode, dtype, method, la.shape[1:], la.shape[0], rb.shape[1:],
                                                rb.shape[0])
                ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
                o = xcorr.correlate(mode, dl, dr, method=method, workspace=ws if ws_bytes else None)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    xcorr.correlate(mode, dl, dr, method=method, out=o, workspace=ws if ws_bytes else None)
                e1.record()
                e1.synchronize()
                ms = e0.elapsed_time(e1) / reps
                host = o.cpu().numpy()
                err = max(oracle.max_rel_to_max(host[k], ref[k]) for k in range(ref.shape[0]))
                row[method] = {"correlations_per_s": ref.shape[0] / (ms / 1000.0), "ms": ms,
                               "max_rel_err_vs_fp64": err}
            out.append(row)
    return out


def reference_gpu_study(torch, xcorr, line, reps=10):
    """Baseline leg: the reference's own nai_shuffle GPU kernels on this GPU
    (compiled unchanged from its sources into oracle/_ref/ by
    oracle/build_ref_gpu.py, launched by oracle/ref_gpu.py with its launchers'
    grid), on the same inputs as the plain kernel: one_to_one 128x128
    (seed 1), the headline one_to_many 256x256 x 64 (seed 2), and 8 + 32 x
    64x64 N(0,1) (seed 3) as n_to_mn and n_to_m, FP32.  Each kernel is timed
    over a small sweep of the reference's own launch arguments
    (benchmarking/args_test/args_test.yml ranges); the fastest is reported
    with its error against FP64.  The n_to_mn / n_to_m forms launch per left
    matrix on 8 streams, as the reference's drivers do (src/n_to_mn.hpp:553-572,
    src/n_to_m.hpp:198-212).  Plain-kernel ("direct") times on the same
    inputs, from this run, stand beside them."""
    from oracle import oracle, ref_gpu

    if not ref_gpu.available():
        return {"unavailable": "reference cubins not built (run oracle/build_ref_gpu.py where the reference is)"}
    R = ref_gpu.RefKernels()
    streams = [torch.cuda.Stream() for _ in range(8)]
    main = torch.cuda.current_stream()

    def time_call(fn, zero=None):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            if zero is not None:
                zero.zero_()
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def per_left(launch, n_left):
        # one launch per left matrix, dealt to 8 streams after the main stream's work
        ev = torch.cuda.Event()
        ev.record(main)
        for i in range(n_left):
            s = streams[i % len(streams)]
            s.wait_event(ev)
            launch(i, s.cuda_stream)
        for s in streams[:n_left]:
            main.wait_stream(s)

    def case(name, mode, left, right, variants, direct_ms):
        n, H, W = left.shape
        m = right.shape[0]
        ref = oracle.run_mode(mode, left, right, dtype="f32acc64", threads=os.cpu_count() or 1)
        if mode == "n_to_mn":  # rights of left l together (the reference's host de-interleave)
            right = np.ascontiguousarray(right.reshape(m // n, n, H, W).transpose(1, 0, 2, 3).reshape(m, H, W))
        dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
        n_out = ref.shape[0]
        out = torch.zeros((n_out, 2 * H - 1, 2 * W - 1), device="cuda")
        rows = []
        for vname, launch, atomic in variants:
            if mode in ("n_to_mn", "n_to_m"):
                # rights of left l: n_to_mn takes rights l, l+n, ... (the reference de-interleaves them first,
                # src/n_to_mn.hpp:165-171; the kernel work is the same on contiguous blocks), n_to_m all M
                k = m // n if mode == "n_to_mn" else m
                osz = (2 * H - 1) * (2 * W - 1)
                fn = lambda launch=launch, k=k: per_left(
                    lambda i, st: launch(dl.data_ptr() + i * H * W * 4,
                                         dr.data_ptr() + (i * k * H * W * 4 if mode == "n_to_mn" else 0),
                                         out.data_ptr() + i * k * osz * 4, k, st), n)
            else:
                fn = lambda launch=launch: launch(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), m,
                                                  main.cuda_stream)
            ms = time_call(fn, out if atomic else None)
            if atomic:
                out.zero_()
                fn()
            torch.cuda.synchronize()
            got = out.cpu().numpy().astype(np.float64)
            if mode == "n_to_mn":  # blocks of left l's rights back to the reference order (output i: left i mod n)
                got = got.reshape(n, m // n, *got.shape[1:]).transpose(1, 0, 2, 3).reshape(got.shape)
            err = max(oracle.max_rel_to_max(got[q], ref[q]) for q in range(n_out))
            rows.append({"kernel": vname, "ms": ms, "correlations_per_s": n_out / (ms / 1000.0),
                         "max_rel_err_vs_fp64": err})
        best = min(rows, key=lambda r: r["ms"])
        return {"config": name, "dtype": "f32", "outputs": int(n_out), "best": best,
                "direct_ms": direct_ms, "direct_speedup_over_best": (best["ms"] / direct_ms) if direct_ms else None,
                "variants": rows}

    def o2m_variants(H, W):
        v = []
        for S in (2, 4):
            for M in (2, 4):
                for Rr in (2, 4):
                    for warps in (4, 8):
                        v.append((f"ccn_shuffle_one_to_many_multirow_both_multimat_right<{S},{M},{Rr}> warps={warps}",
                                  lambda l, r, o, k, st, S=S, M=M, Rr=Rr, warps=warps:
                                  R.one_to_many_multirow_both_multimat_right(l, r, o, H, W, k, warps=warps, shifts=S,
                                                                             mats=M, rows=Rr, stream=st), False))
        return v

    def wd_variants(H, W, mats_list):
        v = []
        for M in mats_list:
            for max_rows in (8, 32):
                v.append((f"ccn_shuffle_multimat_right_work_distribution<{M}, rectangle> warps=8 max_rows={max_rows}",
                          lambda l, r, o, k, st, M=M, max_rows=max_rows:
                          R.multimat_right_work_distribution(l, r, o, H, W, k, warps=8, mats=M, max_rows=max_rows,
                                                             stream=st), True))
        return v

    def direct_ms_of(config, dtype="f32"):
        for row in line.get("configs", []):
            if row["config"] == config and row["dtype"] == dtype:
                return row["direct"]["ms"]
        return None

    out = []
    rng = np.random.default_rng(1)
    a, b = rng.random((1, 128, 128)).astype(np.float32), rng.random((1, 128, 128)).astype(np.float32)
    c1 = [(f"ccn_shuffle warps={w}", lambda l, r, o, k, st, w=w: R.ccn_shuffle(l, r, o, 128, 128, warps=w, stream=st),
           False) for w in (4, 8, 16)]
    c1 += wd_variants(128, 128, (1,))
    out.append(case("one_to_one 128x128 U[0,1) seed 1", "one_to_one", a, b, c1,
                    direct_ms_of("one_to_one 128x128 U[0,1) seed 1")))
    left, right = make_inputs()
    plain = line.get("plain_fp32", {}).get("ms_per_step")
    out.append(case("one_to_many 256x256 x 64 U[0,1) seed 2 (the headline workload)", "one_to_many", left, right,
                    o2m_variants(256, 256) + wd_variants(256, 256, (4, 8)), plain))
    rng = np.random.default_rng(3)
    a = rng.standard_normal((8, 64, 64)).astype(np.float32)
    b = rng.standard_normal((32, 64, 64)).astype(np.float32)
    for mode, cname in (("n_to_mn", "n_to_mn 8+32 x 64x64 N(0,1) seed 3"), ("n_to_m", "n_to_m 8+32 x 64x64 N(0,1) seed 3")):
        out.append(case(cname, mode, a, b, o2m_variants(64, 64) + wd_variants(64, 64, (4,)), direct_ms_of(cname)))
    return out


def gpu_launches(method, steps):
    # kernels per xc_correlate call: direct 1; fft 2 pads + multiply + normalise
    # (+ cuFFT's own); tc: sums; column sums with the means, split planes,
    # accumulation windows and work list; row scans; correction; tcgen05 kernel
    per_step = {"direct": 1, "fft": 4, "tc_bf16x3": 5, "tc_tf32x3": 5}.get(method, 1)
    return per_step * steps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="tc_bf16x3", choices=["direct", "fft", "tc_bf16x3", "tc_tf32x3"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ragged", action="store_true", help="skip the ragged n_to_m side study")
    ap.add_argument("--no-configs", action="store_true", help="skip the other fixed configurations")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the baseline leg that times the reference's own GPU kernels")
    ap.add_argument("--no-csv", action="store_true", help="skip the CSV load/store study of the cross CLI")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
