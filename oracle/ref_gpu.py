"""The reference's own GPU kernels on this GPU: test and measurement
infrastructure, never part of the library.

Loads the cubins that oracle/build_ref_gpu.py compiles from the reference's
unchanged sources (oracle/_ref/*.cubin.gz) through the CUDA driver API and
launches them with the grid and block the reference's host launchers compute,
restated here (the launchers themselves are host code of the reference's
build, which cannot be used on this machine):

  ccn_shuffle<float, float>                                run_ccn_shuffle,
      src/naive_shuffle.cu:452-484: block (32, warps), grid
      (ceil(Sx / 32), ceil(Sy / warps)).
  ccn_shuffle_multimat_right_work_distribution<M, rectangle, float, float>
      ccn_shuffle_multimat_right_work_distribution_right_mats_dispatch,
      src/naive_shuffle_multimat_right.cu:628-703: block (32, warps), grid
      (ceil(Sx / 32) * ceil(n_right / M), ceil(workers / warps)) with
      workers = Sy * ceil(H / max_rows) (rectangle_distribution::num_workers,
      src/row_distribution.cuh:222-228); adds into a zeroed output.
  ccn_shuffle_one_to_many_multirow_both_multimat_right<S, M, R, float, float>
      ..._left_rows_dispatch, src/naive_shuffle_one_to_many_multirow_both_multimat_right.cu:582-631:
      block (32, warps), grid (ceil(Sx / 32) * ceil(n_right / M),
      ceil(Sy / (warps * S))); writes its output.

Kernels are found by their names (the module's functions are enumerated and
matched on the kernel name and its template arguments).  Equal-size inputs
only, as in the reference: matrix_size = (W, H), search_size = (2W-1, 2H-1).
"""
from __future__ import annotations

import ctypes
import gzip
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
UNITS = ["naive_shuffle", "naive_shuffle_multimat_right", "naive_shuffle_one_to_many_multirow_both_multimat_right"]


class _Size2(ctypes.Structure):  # the reference's dsize2_t (src/types.cuh:12-156): {x, y} of unsigned
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint)]


def available() -> bool:
    return all(os.path.exists(os.path.join(REF, u + ".cubin.gz")) for u in UNITS)


def _div_up(a: int, b: int) -> int:
    return (a + b - 1) // b


class RefKernels:
    """The reference kernels loaded into the current CUDA context (torch's)."""

    def __init__(self):
        import torch

        torch.zeros(1, device="cuda")  # the primary context is current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        c = ctypes
        self.cu.cuCtxGetCurrent.argtypes = [c.POINTER(c.c_void_p)]
        self.cu.cuModuleLoadData.argtypes = [c.POINTER(c.c_void_p), c.c_void_p]
        self.cu.cuModuleGetFunctionCount.argtypes = [c.POINTER(c.c_uint), c.c_void_p]
        self.cu.cuModuleEnumerateFunctions.argtypes = [c.POINTER(c.c_void_p), c.c_uint, c.c_void_p]
        self.cu.cuFuncGetName.argtypes = [c.POINTER(c.c_char_p), c.c_void_p]
        self.cu.cuLaunchKernel.argtypes = [c.c_void_p, c.c_uint, c.c_uint, c.c_uint, c.c_uint, c.c_uint, c.c_uint,
                                           c.c_uint, c.c_void_p, c.POINTER(c.c_void_p), c.POINTER(c.c_void_p)]
        ctx = c.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(c.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.funcs = {}  # name -> CUfunction
        self._images = []
        for unit in UNITS:
            with gzip.open(os.path.join(REF, unit + ".cubin.gz"), "rb") as f:
                image = ctypes.create_string_buffer(f.read())
            self._images.append(image)
            mod = c.c_void_p()
            self._check(self.cu.cuModuleLoadData(c.byref(mod), c.cast(image, c.c_void_p)), "cuModuleLoadData")
            n = c.c_uint()
            self._check(self.cu.cuModuleGetFunctionCount(c.byref(n), mod), "cuModuleGetFunctionCount")
            fns = (c.c_void_p * n.value)()
            self._check(self.cu.cuModuleEnumerateFunctions(fns, n.value, mod), "cuModuleEnumerateFunctions")
            for fn in fns:
                name = c.c_char_p()
                self._check(self.cu.cuFuncGetName(c.byref(name), fn), "cuFuncGetName")
                self.funcs[name.value.decode()] = fn

    @staticmethod
    def _check(res, what):
        if res != 0:
            raise RuntimeError(f"{what} failed with CUresult {res}")

    def find(self, *parts: str):
        hits = [fn for name, fn in self.funcs.items() if all(p in name for p in parts)]
        if len(hits) != 1:
            raise KeyError(f"{len(hits)} kernels match {parts}")
        return hits[0]

    def _launch(self, fn, grid, block, args, stream):
        c = ctypes
        holders = []
        for a in args:
            holders.append(a if isinstance(a, (c.Structure, c._SimpleCData)) else c.c_void_p(a))
        params = (c.c_void_p * len(holders))(*[c.cast(c.byref(h), c.c_void_p) for h in holders])
        self._check(self.cu.cuLaunchKernel(fn, grid[0], grid[1], 1, block[0], block[1], 1, 0, c.c_void_p(stream),
                                           params, None), "cuLaunchKernel")

    # ---- launchers (FP32, equal sizes H x W, n_right right matrices) ----
    def ccn_shuffle(self, left, right, out, H, W, warps=8, stream=0):
        Sy, Sx = 2 * H - 1, 2 * W - 1
        fn = self.find("ccn_shuffleIffEEv")
        self._launch(fn, (_div_up(Sx, 32), _div_up(Sy, warps)), (32, warps),
                     [left, right, out, _Size2(W, H), _Size2(Sx, Sy)], stream)

    def multimat_right_work_distribution(self, left, right, out, H, W, n_right, warps=8, mats=1, max_rows=16,
                                         stream=0):
        """Adds into `out` (zero it first)."""
        Sy, Sx = 2 * H - 1, 2 * W - 1
        fn = self.find(f"ccn_shuffle_multimat_right_work_distributionILj{mats}ENS_22rectangle_distributionEffE")
        workers = Sy * _div_up(H, max_rows)
        self._launch(fn, (_div_up(Sx, 32) * _div_up(n_right, mats), _div_up(workers, warps)), (32, warps),
                     [left, right, out, _Size2(W, H), _Size2(Sx, Sy), ctypes.c_uint(n_right),
                      ctypes.c_uint(max_rows)], stream)

    def one_to_many_multirow_both_multimat_right(self, left, right, out, H, W, n_right, warps=8, shifts=4, mats=4,
                                                 rows=4, stream=0):
        Sy, Sx = 2 * H - 1, 2 * W - 1
        fn = self.find(f"ccn_shuffle_one_to_many_multirow_both_multimat_rightILj{shifts}ELj{mats}ELj{rows}EffE")
        self._launch(fn, (_div_up(Sx, 32) * _div_up(n_right, mats), _div_up(Sy, warps * shifts)), (32, warps),
                     [left, right, out, _Size2(W, H), _Size2(Sx, Sy), ctypes.c_uint(n_right)], stream)
