"""Build the GB300 library, the `cross` CLI and (as test infrastructure) the
CPU oracle, in tree.

Outputs (git-ignored):
  cross-corr_gb300/_build/libxcorr.so   CUDA kernels + C ABI (sm_103a only)
  cross-corr_gb300/_build/cross         the reference-compatible CLI
  oracle/_build/libxcorr_oracle.so      CPU oracle (tests, smoke, cpu baseline)

No cmake: one nvcc invocation per translation unit, run in parallel, then a
link step.  The same commands work on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]
CUDA_SOURCES = ["xc_runtime.cu", "direct_simt.cu", "ragged.cu", "fft_glue.cu", "fft_pipeline.cu", "tc_bf16x3.cu",
                "mlp.cu", "api.cu"]
CLI_SOURCES = ["main.cpp", "data_array.cpp", "json_args.cpp", "algorithms.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    return hs


def build_library(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    heads = _headers()
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + heads):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + list(extra_flags or []) + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    lib = os.path.join(OUT, "libxcorr.so")
    if _stale(lib, objs):
        cuda_lib = os.path.join(_cuda_home(), "lib64")
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs +
             ["-L" + cuda_lib, "-lcufft", "-lcudart", "-Xlinker", "-rpath=" + cuda_lib], verbose)
    return lib


def build_cli(verbose: bool = False) -> str:
    lib = os.path.join(OUT, "libxcorr.so")
    exe = os.path.join(OUT, "cross")
    srcs = [os.path.join(CLI, s) for s in CLI_SOURCES]
    heads = [os.path.join(CLI, f) for f in os.listdir(CLI) if f.endswith(".hpp")] + [os.path.join(INCLUDE, "xcorr.h")]
    if _stale(exe, srcs + heads + [lib]):
        cuda = _cuda_home()
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), "-o", exe] +
             srcs + ["-L" + OUT, "-lxcorr", "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lpthread",
                     "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")], verbose)
    return exe


def build_oracle(verbose: bool = False) -> str:
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], verbose)
    return os.path.join(ROOT, "oracle", "_build", "libxcorr_oracle.so")


def build_all(verbose: bool = False) -> None:
    build_oracle(verbose)
    build_library(verbose)
    build_cli(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", OUT)
