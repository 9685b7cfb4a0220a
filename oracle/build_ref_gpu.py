"""Recipe: the reference's own GPU kernels as sm_103a cubins (test and
measurement infrastructure, not part of the library).

Compiles, unchanged and where they lie in the reference checkout, the device
code of three reference translation units with nvcc -cubin:

  src/naive_shuffle.cu                                    ccn_shuffle, ccn_shuffle_work_distribution
  src/naive_shuffle_multimat_right.cu                     ccn_shuffle_multimat_right[_work_distribution]
  src/naive_shuffle_one_to_many_multirow_both_multimat_right.cu
                                                          the reference's best one_to_many kernel

with the algorithm limits of its release build (CMakeLists.txt:16-43).  The
outputs go to oracle/_ref/ only, gzip-compressed (the one_to_many unit
instantiates every tile combination up to its limits for int, float and
double: 130 MB of cubin, 17 MB compressed).  The host side that launches them
is oracle/ref_gpu.py.  The reference's own CMake build is not used.

Usage: python oracle/build_ref_gpu.py [reference checkout, default
/root/reference].  Takes about 12 minutes (the one_to_many unit); does
nothing when the outputs are newer than their sources.
"""
from __future__ import annotations

import concurrent.futures as cf
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
UNITS = ["naive_shuffle", "naive_shuffle_multimat_right", "naive_shuffle_one_to_many_multirow_both_multimat_right"]
# release values of the reference's ALG_LIMIT_OPTIONS (CMakeLists.txt:16-43)
LIMITS = {
    "SHUFFLE_MULTIMAT_RIGHT_RIGHT_MATRICES_PER_THREAD_LIMIT": 8,
    "SHUFFLE_ONE_TO_MANY_MULTIROW_BOTH_MULTIMAT_RIGHT_SHIFTS_PER_RIGHT_MATRIX_LIMIT": 4,
    "SHUFFLE_ONE_TO_MANY_MULTIROW_BOTH_MULTIMAT_RIGHT_RIGHT_MATRICES_PER_THREAD_LIMIT": 4,
    "SHUFFLE_ONE_TO_MANY_MULTIROW_BOTH_MULTIMAT_RIGHT_LEFT_ROWS_PER_ITERATION_LIMIT": 4,
}


def build(ref_root: str = "/root/reference", verbose: bool = True) -> list:
    src = os.path.join(ref_root, "src")
    if not os.path.isdir(src):
        raise SystemExit(f"no reference sources at {src}")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT, exist_ok=True)
    defs = [f"-D{k}={v}" for k, v in LIMITS.items()]

    def one(unit):
        cu = os.path.join(src, unit + ".cu")
        dst = os.path.join(OUT, unit + ".cubin.gz")
        if os.path.exists(dst) and os.path.getmtime(dst) > os.path.getmtime(cu):
            return dst
        with tempfile.TemporaryDirectory() as tmp:
            cubin = os.path.join(tmp, unit + ".cubin")
            cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-I" + src,
                   *defs, cu, "-o", cubin]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{' '.join(cmd)}\n{r.stderr[-2000:]}")
            with open(cubin, "rb") as f, gzip.open(dst + ".tmp", "wb", compresslevel=6) as g:
                shutil.copyfileobj(f, g)
            os.replace(dst + ".tmp", dst)
        if verbose:
            print("built", dst, flush=True)
        return dst

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        return list(ex.map(one, UNITS))


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
