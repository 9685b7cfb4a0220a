"""Python face of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/libxcorr_oracle.so`` (built from ``xcorr_oracle.c`` by
``__graft_entry__.build()`` or ``make -C oracle``) and exposes the reference's
CPU algorithms on numpy arrays.  Only tests, the smoke check and the CPU
baseline leg of ``bench.py`` import this module; the product library never does.

Restated reference behaviour (file:line in MK4H/cross-corr):
  * ``run_mode``      -- cpu_cross_corr_* (src/validate.hpp:216-298)
  * ``validate``      -- validate_result (src/validate.hpp:134-188)
  * ``normalize_fft`` -- normalize_fft_results (src/fft_helpers.hpp:193-261)
  * ``read_csv`` / ``write_csv`` -- data_array CSV format
    (src/matrix.hpp:94-185; header ``# rows,cols,count``, matrices stacked)
  * ``interleaved_index`` -- get_interleaved_index (src/matrix.hpp:614-618)
"""
from __future__ import annotations

import ctypes
import gzip
import io
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libxcorr_oracle.so")

MODES = {"one_to_one": 0, "one_to_many": 1, "n_to_mn": 2, "n_to_m": 3}
DTYPES = {"f32": 0, "f64": 1, "f32acc64": 2}

_lib = None


def build() -> str:
    """Compile the oracle with the committed Makefile (plain gcc)."""
    import subprocess

    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i, l = ctypes.c_void_p, ctypes.c_int, ctypes.c_long
        L.xco_run_mode.argtypes = [i, i, vp, i, i, i, vp, i, i, i, vp, i]
        L.xco_run_mode.restype = i
        L.xco_num_outputs.argtypes = [i, i, i]
        L.xco_num_outputs.restype = l
        L.xco_run_pairs.argtypes = [i, i, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i]
        L.xco_run_pairs.restype = i
        dp = ctypes.POINTER(ctypes.c_double)
        L.xco_validate.argtypes = [vp, vp, ctypes.c_size_t, dp, dp, dp, dp, dp]
        L.xco_validate.restype = None
        L.xco_normalize_fft.argtypes = [vp, i, i, vp]
        L.xco_normalize_fft.restype = None
        L.xco_interleaved_index.argtypes = [l, l, l]
        L.xco_interleaved_index.restype = l
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def num_outputs(mode: str, n_left: int, n_right: int) -> int:
    return int(lib().xco_num_outputs(MODES[mode], n_left, n_right))


def pair_of_output(mode: str, n_left: int, n_right: int, o: int):
    """(left, right) indices of output ``o`` in the reference's result order."""
    if mode == "n_to_mn":
        return o % n_left, o
    if mode == "n_to_m":
        return o // n_right, o % n_right
    if mode == "one_to_many":
        return 0, o
    return 0, 0


def run_mode(mode: str, left: np.ndarray, right: np.ndarray, dtype: str = "f32acc64",
             threads: int = 1) -> np.ndarray:
    """Correlate stacked matrices ``left`` (n,Hl,Wl) and ``right`` (m,Hr,Wr).

    dtype ``f32``: float accumulate (reference T=float); ``f64``: double;
    ``f32acc64``: float inputs accumulated and returned in double (FP64 oracle).
    """
    if left.ndim == 2:
        left = left[None]
    if right.ndim == 2:
        right = right[None]
    tin = np.float64 if dtype == "f64" else np.float32
    tout = np.float32 if dtype == "f32" else np.float64
    left = np.ascontiguousarray(left, dtype=tin)
    right = np.ascontiguousarray(right, dtype=tin)
    n, hl, wl = left.shape
    m, hr, wr = right.shape
    n_out = num_outputs(mode, n, m)
    if n_out < 0:
        raise ValueError(f"invalid matrix counts for {mode}: {n} left, {m} right")
    out = np.empty((n_out, hl + hr - 1, wl + wr - 1), dtype=tout)
    rc = lib().xco_run_mode(MODES[mode], DTYPES[dtype], _ptr(left), n, hl, wl, _ptr(right), m, hr, wr,
                            _ptr(out), int(threads))
    if rc != 0:
        raise ValueError("oracle rejected the inputs")
    return out


def correlate(left: np.ndarray, right: np.ndarray, dtype: str = "f32acc64") -> np.ndarray:
    """Full correlation of one pair (scipy correlate2d(left, right) order)."""
    return run_mode("one_to_one", left, right, dtype)[0]


def run_pairs(lefts: Sequence[np.ndarray], rights: Sequence[np.ndarray], dtype: str = "f32acc64",
              threads: int = 1):
    """Ragged pair list: returns one output array per (lefts[p], rights[p])."""
    tin = np.float64 if dtype == "f64" else np.float32
    tout = np.float32 if dtype == "f32" else np.float64
    n = len(lefts)
    hl = np.array([a.shape[0] for a in lefts], dtype=np.int32)
    wl = np.array([a.shape[1] for a in lefts], dtype=np.int32)
    hr = np.array([a.shape[0] for a in rights], dtype=np.int32)
    wr = np.array([a.shape[1] for a in rights], dtype=np.int32)
    lsz = (hl.astype(np.int64) * wl)
    rsz = (hr.astype(np.int64) * wr)
    osz = (hl + hr - 1).astype(np.int64) * (wl + wr - 1)
    loff = np.concatenate([[0], np.cumsum(lsz)[:-1]]).astype(np.int64)
    roff = np.concatenate([[0], np.cumsum(rsz)[:-1]]).astype(np.int64)
    ooff = np.concatenate([[0], np.cumsum(osz)[:-1]]).astype(np.int64)
    L = np.concatenate([np.asarray(a, dtype=tin).ravel() for a in lefts])
    R = np.concatenate([np.asarray(a, dtype=tin).ravel() for a in rights])
    out = np.empty(int(osz.sum()), dtype=tout)
    lib().xco_run_pairs(DTYPES[dtype], n, _ptr(hl), _ptr(wl), _ptr(hr), _ptr(wr), _ptr(loff), _ptr(roff),
                        _ptr(ooff), _ptr(L), _ptr(R), _ptr(out), int(threads))
    res = []
    for p in range(n):
        res.append(out[ooff[p]:ooff[p] + osz[p]].reshape(hl[p] + hr[p] - 1, wl[p] + wr[p] - 1))
    return res


def validate(result: np.ndarray, valid: np.ndarray) -> dict:
    """validate_result: Max/Mean/Stddev of the element-wise relative difference."""
    a = np.ascontiguousarray(result, dtype=np.float64).ravel()
    b = np.ascontiguousarray(valid, dtype=np.float64).ravel()
    if a.size != b.size:
        raise ValueError("Cannot validate matrices of different sizes")
    vals = [ctypes.c_double() for _ in range(5)]
    lib().xco_validate(_ptr(a), _ptr(b), a.size, *[ctypes.byref(v) for v in vals])
    return {"max": vals[0].value, "mean": vals[1].value, "stddev": vals[2].value,
            "at_result": vals[3].value, "at_valid": vals[4].value}


def max_rel_to_max(result: np.ndarray, oracle64: np.ndarray) -> float:
    """max|out - oracle| / max|oracle| for one output matrix (the accuracy gate)."""
    o = np.asarray(oracle64, dtype=np.float64)
    d = np.abs(np.asarray(result, dtype=np.float64) - o).max()
    m = np.abs(o).max()
    return float(d / m) if m > 0 else float(d)


def normalize_fft(res: np.ndarray) -> np.ndarray:
    """normalize_fft_results on a stack (k,Py,Px) of raw circular correlations."""
    res = np.ascontiguousarray(res, dtype=np.float64)
    if res.ndim == 2:
        res = res[None]
    k, py, px = res.shape
    out = np.empty((k, py - 1, px - 1), dtype=np.float64)
    for i in range(k):
        lib().xco_normalize_fft(_ptr(res[i]), py, px, _ptr(out[i]))
    return out


def interleaved_index(idx: int, group_size: int, num_groups: int) -> int:
    return int(lib().xco_interleaved_index(idx, group_size, num_groups))


# --------------------------------------------------------------------------
# CSV format of data_array (src/matrix.hpp:94-185)
# --------------------------------------------------------------------------
def read_csv(path: str, dtype=np.float64) -> np.ndarray:
    """Read ``# rows,cols,count`` + stacked row-major matrices -> (count,rows,cols)."""
    opener = gzip.open if path.endswith(".gz") else open
    with opener(path, "rt") as f:
        header = f.readline()
        if not header.startswith("# "):
            raise ValueError("Invalid file header format")
        parts = [int(p) for p in header[2:].strip().split(",")]
        rows, cols = parts[0], parts[1]
        count = parts[2] if len(parts) > 2 else 1
        data = np.loadtxt(io.StringIO(f.read()), delimiter=",", dtype=dtype, ndmin=2)
    return data.reshape(count, rows, cols)


def write_csv(path: str, mats: np.ndarray, fmt: str = "%.17g") -> None:
    mats = np.asarray(mats)
    if mats.ndim == 2:
        mats = mats[None]
    k, rows, cols = mats.shape
    with open(path, "w") as f:
        f.write(f"# {rows},{cols},{k}\n")
        np.savetxt(f, mats.reshape(k * rows, cols), delimiter=",", fmt=fmt)
