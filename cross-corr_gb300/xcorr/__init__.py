"""Python binding of the GB300 cross-correlation library (ctypes over the C ABI).

The library itself is ``cross-corr_gb300/_build/libxcorr.so`` (CUDA kernels and
the C ABI of ``include/xcorr.h``); this module only marshals arguments.  Device
buffers come from PyTorch (CUDA tensors) or numpy arrays for the host-buffer
entry point.  Importing never falls back to anything else: if the library has
not been built, every call raises ``LibraryNotBuilt``.

Mode / result-order conventions follow the reference (src/validate.hpp:216-298):
  one_to_one : 1 x 1 -> 1;  one_to_many: 1 x M -> M (output i = right i)
  n_to_mn    : n x (m*n) -> m*n (output i = left i mod n with right i)
  n_to_m     : n x M -> n*M (output l*M + r = left l with right r)
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libxcorr.so")
CLI_PATH = os.path.join(PKG, "_build", "cross")

MODES = {"one_to_one": 0, "one_to_many": 1, "n_to_mn": 2, "n_to_m": 3}
DTYPES = {"f32": 0, "f64": 1}
METHODS = {"auto": 0, "direct": 1, "fft": 2, "tc_bf16x3": 3, "tc_tf32x3": 4}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "cuFFT error", 4: "unsupported",
          5: "workspace too small", 6: "device wait timed out"}

# Every symbol declared in include/xcorr.h (checked by the CPU test suite).
EXPORTED = [
    "xc_version", "xc_status_string", "xc_last_error", "xc_device_check", "xc_check_device",
    "xc_debug_expire_wait", "xc_kernel_timing", "xc_kernel_timing_read", "xc_output_count", "xc_output_size",
    "xc_workspace_size", "xc_correlate", "xc_correlate_host", "xc_correlate_host_async", "xc_host_wait",
    "xc_release_thread_cache", "xc_correlate_tc_noalloc",
    "xc_fft_plan_create", "xc_fft_plan_workspace_size", "xc_fft_plan_pad_size", "xc_fft_execute",
    "xc_fft_forward", "xc_fft_multiply", "xc_fft_inverse", "xc_fft_plan_destroy",
    "xc_run_ccn_shuffle_f32", "xc_run_ccn_shuffle_f64",
    "xc_run_ccn_shuffle_multimat_right_f32", "xc_run_ccn_shuffle_multimat_right_f64",
    "xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f32",
    "xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_f64",
    "xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_f32",
    "xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_f64",
    "xc_run_ccn_shuffle_work_distribution_f32", "xc_run_ccn_shuffle_work_distribution_f64",
    "xc_run_ccn_shuffle_multimat_right_work_distribution_f32",
    "xc_run_ccn_shuffle_multimat_right_work_distribution_f64",
    "xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_f32",
    "xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_f64",
    "xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem_f32",
    "xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution_local_mem_f64",
    "xc_run_ccn_shuffle_multirow_right_f32", "xc_run_ccn_shuffle_multirow_right_f64",
    "xc_run_ccn_shuffle_multirow_both_f32", "xc_run_ccn_shuffle_multirow_both_f64",
    "xc_run_ccn_shuffle_multirow_both_local_mem_f32", "xc_run_ccn_shuffle_multirow_both_local_mem_f64",
    "xc_run_ccn_shuffle_multirow_right_multimat_right_f32", "xc_run_ccn_shuffle_multirow_right_multimat_right_f64",
    "xc_run_hadamard_original_c64", "xc_run_hadamard_original_c128",
    "xc_run_hadamard_n_to_m_over_output_c64", "xc_run_hadamard_n_to_m_over_output_c128",
    "xc_run_scatter_f32", "xc_run_scatter_f64",
    "xc_normalize_fft_results_f32", "xc_normalize_fft_results_f64",
    "xc_ragged_plan_create", "xc_ragged_autotune", "xc_ragged_execute", "xc_ragged_plan_destroy",
    "xc_ragged_describe", "xc_ragged_select",
    "xc_correlate_pairs", "xc_selector_features", "xc_mlp_forward", "xc_mlp_gradient", "xc_mlp_adam_step",
    "xc_selector_load", "xc_selector_load_builtin", "xc_select_method", "xc_autotune_method",
    "xc_algorithm", "xc_select_algorithm", "xc_correlate_algo", "xc_time_algorithm", "xc_autotune_algorithm",
]


class LibraryNotBuilt(RuntimeError):
    pass


class XcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Size2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint32), ("y", ctypes.c_uint32)]


class Algo(ctypes.Structure):
    """xc_algo: a method and one of its tile configurations."""
    _fields_ = [("method", ctypes.c_int), ("tile", ctypes.c_int32)]


class MatrixDesc(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint64), ("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32)]


class PairDesc(ctypes.Structure):
    _fields_ = [("left", ctypes.c_uint32), ("right", ctypes.c_uint32), ("out_offset", ctypes.c_uint64)]


class RaggedVariant(ctypes.Structure):
    _fields_ = [("index", ctypes.c_int32), ("n_variants", ctypes.c_int32), ("tile_shape", ctypes.c_int32),
                ("tc_pairs", ctypes.c_uint32), ("tc_min_macs", ctypes.c_uint64)]


def size2(rows: int, cols: int) -> Size2:
    return Size2(int(cols), int(rows))


_lib = None


def lib():
    """Load libxcorr.so (raises LibraryNotBuilt when it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryNotBuilt(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        c = ctypes
        vp, u32, i, sz = c.c_void_p, c.c_uint32, c.c_int, c.c_size_t
        L.xc_version.restype = c.c_char_p
        L.xc_status_string.restype = c.c_char_p
        L.xc_status_string.argtypes = [i]
        L.xc_last_error.restype = c.c_char_p
        L.xc_device_check.argtypes = [i]
        L.xc_check_device.argtypes = [vp]
        L.xc_debug_expire_wait.argtypes = [u32, vp]
        L.xc_kernel_timing.argtypes = [i]
        L.xc_kernel_timing_read.argtypes = [c.POINTER(c.c_double), c.POINTER(u32)]
        L.xc_output_count.argtypes = [i, u32, u32, c.POINTER(c.c_uint64)]
        L.xc_output_size.argtypes = [Size2, Size2, c.POINTER(Size2)]
        L.xc_workspace_size.argtypes = [i, i, i, Size2, u32, Size2, u32, c.POINTER(sz)]
        L.xc_correlate.argtypes = [i, i, i, vp, Size2, u32, vp, Size2, u32, vp, vp, sz, vp]
        L.xc_correlate_host.argtypes = [i, i, i, vp, Size2, u32, vp, Size2, u32, vp, vp]
        L.xc_correlate_host_async.argtypes = [i, i, i, vp, Size2, u32, vp, Size2, u32, vp, vp,
                                              c.POINTER(c.c_uint64)]
        L.xc_host_wait.argtypes = [c.c_uint64]
        L.xc_release_thread_cache.restype = None
        L.xc_correlate_tc_noalloc.argtypes = [i, vp, Size2, u32, vp, Size2, u32, vp, vp]
        L.xc_fft_plan_create.argtypes = [c.POINTER(vp), i, i, Size2, u32, Size2, u32, Size2]
        L.xc_fft_plan_workspace_size.argtypes = [vp, c.POINTER(sz)]
        L.xc_fft_plan_pad_size.argtypes = [vp, c.POINTER(Size2)]
        L.xc_fft_execute.argtypes = [vp, vp, vp, vp, i, vp, sz, vp]
        L.xc_fft_forward.argtypes = [vp, vp, vp, vp, sz, vp]
        L.xc_fft_multiply.argtypes = [vp, vp, sz, vp]
        L.xc_fft_inverse.argtypes = [vp, vp, i, vp, sz, vp]
        L.xc_fft_plan_destroy.argtypes = [vp]
        P = c.POINTER
        L.xc_ragged_plan_create.argtypes = [P(vp), i, vp, P(MatrixDesc), u32, vp, P(MatrixDesc), u32, P(PairDesc),
                                            u32, vp]
        L.xc_ragged_autotune.argtypes = [vp, vp, P(c.c_int), P(c.c_double)]
        L.xc_ragged_execute.argtypes = [vp, vp]
        L.xc_ragged_describe.argtypes = [vp, i, P(RaggedVariant)]
        L.xc_ragged_select.argtypes = [vp, i]
        L.xc_ragged_plan_destroy.argtypes = [vp]
        L.xc_correlate_pairs.argtypes = [i, vp, P(MatrixDesc), u32, vp, P(MatrixDesc), u32, P(PairDesc), u32, vp,
                                         vp]
        f32p = P(c.c_float)
        L.xc_selector_features.argtypes = [i, Size2, u32, Size2, u32, f32p]
        L.xc_mlp_forward.argtypes = [vp, vp, u32, vp, vp]
        L.xc_mlp_gradient.argtypes = [vp, vp, vp, vp, u32, c.c_float, vp, vp, vp]
        L.xc_mlp_adam_step.argtypes = [vp, vp, vp, vp, u32, c.c_float, vp]
        L.xc_selector_load.argtypes = [vp]
        L.xc_select_method.argtypes = [i, i, Size2, u32, Size2, u32, P(i)]
        L.xc_autotune_method.argtypes = [i, i, vp, Size2, u32, vp, Size2, u32, vp, vp, P(i), P(c.c_double)]
        L.xc_algorithm.argtypes = [u32, P(Algo)]
        L.xc_select_algorithm.argtypes = [i, i, Size2, u32, Size2, u32, P(Algo)]
        L.xc_correlate_algo.argtypes = [i, i, Algo, vp, Size2, u32, vp, Size2, u32, vp, vp, sz, vp]
        L.xc_time_algorithm.argtypes = [i, i, Algo, vp, Size2, u32, vp, Size2, u32, vp, vp, sz, u32, vp,
                                        P(c.c_double)]
        L.xc_autotune_algorithm.argtypes = [i, i, vp, Size2, u32, vp, Size2, u32, vp, vp, P(Algo), P(c.c_double)]
        for t in ("f32", "f64"):
            getattr(L, f"xc_run_ccn_shuffle_{t}").argtypes = [vp, vp, vp, Size2, Size2, u32, vp]
            getattr(L, f"xc_run_ccn_shuffle_multimat_right_{t}").argtypes = [vp, vp, vp, Size2, Size2, u32, u32, u32,
                                                                              vp]
            getattr(L, f"xc_run_ccn_shuffle_one_to_many_multirow_both_multimat_right_{t}").argtypes = [
                vp, vp, vp, Size2, Size2, u32, u32, u32, u32, u32, vp]
            getattr(L, f"xc_run_ccn_n_to_m_shuffle_multirow_both_multimat_both_{t}").argtypes = [
                vp, vp, vp, Size2, Size2, u32, u32, u32, u32, u32, u32, u32, vp]
            getattr(L, f"xc_run_ccn_shuffle_work_distribution_{t}").argtypes = [vp, vp, vp, Size2, Size2, u32, u32, i,
                                                                                 vp]
            getattr(L, f"xc_run_ccn_shuffle_multimat_right_work_distribution_{t}").argtypes = [
                vp, vp, vp, Size2, Size2, u32, u32, u32, u32, i, vp]
            for lm in ("", "_local_mem"):
                getattr(L, f"xc_run_ccn_shuffle_n_to_m_multimat_both_work_distribution{lm}_{t}").argtypes = [
                    vp, vp, vp, Size2, Size2, u32, u32, u32, u32, u32, u32, i, vp]
                getattr(L, f"xc_run_ccn_shuffle_multirow_both{lm}_{t}").argtypes = [vp, vp, vp, Size2, Size2, u32, u32,
                                                                                    u32, vp]
            getattr(L, f"xc_run_ccn_shuffle_multirow_right_{t}").argtypes = [vp, vp, vp, Size2, Size2, u32, u32, vp]
            getattr(L, f"xc_run_ccn_shuffle_multirow_right_multimat_right_{t}").argtypes = [
                vp, vp, vp, Size2, Size2, u32, u32, u32, u32, vp]
            getattr(L, f"xc_run_scatter_{t}").argtypes = [vp, vp, Size2, u32, Size2, Size2, u32, u32, vp]
            getattr(L, f"xc_normalize_fft_results_{t}").argtypes = [vp, vp, Size2, u32, vp]
        for t in ("c64", "c128"):
            getattr(L, f"xc_run_hadamard_original_{t}").argtypes = [vp, vp, Size2, u32, u32, u32, vp]
            getattr(L, f"xc_run_hadamard_n_to_m_over_output_{t}").argtypes = [vp, vp, vp, Size2, u32, u32, u32, u32,
                                                                               vp]
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise XcError(status, lib().xc_last_error().decode())


def output_count(mode: str, n_left: int, n_right: int) -> int:
    n = ctypes.c_uint64()
    check(lib().xc_output_count(MODES[mode], n_left, n_right, ctypes.byref(n)))
    return int(n.value)


def workspace_size(mode, dtype, method, left_shape, n_left, right_shape, n_right) -> int:
    b = ctypes.c_size_t()
    check(lib().xc_workspace_size(MODES[mode], DTYPES[dtype], METHODS[method], size2(*left_shape), n_left,
                                  size2(*right_shape), n_right, ctypes.byref(b)))
    return int(b.value)


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return int(stream)


def correlate(mode: str, left, right, method: str = "direct", out=None, workspace=None, stream=None):
    """Correlate CUDA tensors ``left`` (n,Hl,Wl) and ``right`` (m,Hr,Wr) on the device.

    ``method`` is a method name or ``"method:tile"`` (xc_correlate_algo).
    Returns the (n_out, Hl+Hr-1, Wl+Wr-1) output tensor.  ``workspace`` (a uint8
    CUDA tensor) is allocated when not given and the method needs one.
    """
    import torch

    if left.dim() == 2:
        left = left.unsqueeze(0)
    if right.dim() == 2:
        right = right.unsqueeze(0)
    if not (left.is_cuda and right.is_cuda):
        raise ValueError("correlate() takes CUDA tensors; use correlate_host() for host arrays")
    dtype = {torch.float32: "f32", torch.float64: "f64"}[left.dtype]
    left = left.contiguous()
    right = right.contiguous()
    n, hl, wl = left.shape
    m, hr, wr = right.shape
    n_out = output_count(mode, n, m)
    if out is None:
        out = torch.empty((n_out, hl + hr - 1, wl + wr - 1), dtype=left.dtype, device=left.device)
    base, _, tile = method.partition(":")
    ws_bytes = workspace_size(mode, dtype, base, (hl, wl), n, (hr, wr), m)
    if ws_bytes and (workspace is None or workspace.numel() < ws_bytes):
        workspace = torch.empty(ws_bytes, dtype=torch.uint8, device=left.device)
    wptr = workspace.data_ptr() if (workspace is not None and ws_bytes) else None
    if tile:
        check(lib().xc_correlate_algo(MODES[mode], DTYPES[dtype], Algo(METHODS[base], int(tile)), left.data_ptr(),
                                      size2(hl, wl), n, right.data_ptr(), size2(hr, wr), m, out.data_ptr(), wptr,
                                      ws_bytes, _stream_ptr(stream)))
    else:
        check(lib().xc_correlate(MODES[mode], DTYPES[dtype], METHODS[base], left.data_ptr(), size2(hl, wl), n,
                                 right.data_ptr(), size2(hr, wr), m, out.data_ptr(), wptr, ws_bytes,
                                 _stream_ptr(stream)))
    return out


def correlate_host(mode: str, left: np.ndarray, right: np.ndarray, method: str = "direct", out=None, stream=None):
    """Host arrays in, host array out (H2D, correlation, D2H inside the call)."""
    if left.ndim == 2:
        left = left[None]
    if right.ndim == 2:
        right = right[None]
    dtype = "f64" if left.dtype == np.float64 else "f32"
    npdt = np.float64 if dtype == "f64" else np.float32
    left = np.ascontiguousarray(left, dtype=npdt)
    right = np.ascontiguousarray(right, dtype=npdt)
    n, hl, wl = left.shape
    m, hr, wr = right.shape
    n_out = output_count(mode, n, m)
    if out is None:
        out = np.empty((n_out, hl + hr - 1, wl + wr - 1), dtype=npdt)
    check(lib().xc_correlate_host(MODES[mode], DTYPES[dtype], METHODS[method], left.ctypes.data, size2(hl, wl), n,
                                  right.ctypes.data, size2(hr, wr), m, out.ctypes.data,
                                  None if stream is None else int(stream)))
    return out


def correlate_host_async(mode: str, left: np.ndarray, right: np.ndarray, out: np.ndarray, method: str = "direct",
                         stream=None) -> int:
    """Enqueue a host-buffer correlation (xc_correlate_host_async) and return
    its ticket; `left`, `right` and `out` are C-contiguous arrays of the
    problem's dtype (pinned memory lets the copies overlap kernels) that must
    stay alive, and `out` unread, until ``host_wait(ticket)``."""
    n, hl, wl = left.shape
    m, hr, wr = right.shape
    dtype = "f64" if left.dtype == np.float64 else "f32"
    for a in (left, right, out):
        if not a.flags["C_CONTIGUOUS"] or a.dtype != left.dtype:
            raise ValueError("left, right and out must be C-contiguous arrays of one dtype")
    if out.shape != (output_count(mode, n, m), hl + hr - 1, wl + wr - 1):
        raise ValueError("out has the wrong shape")
    t = ctypes.c_uint64()
    check(lib().xc_correlate_host_async(MODES[mode], DTYPES[dtype], METHODS[method], left.ctypes.data,
                                        size2(hl, wl), n, right.ctypes.data, size2(hr, wr), m, out.ctypes.data,
                                        None if stream is None else int(stream), ctypes.byref(t)))
    return t.value


def host_wait(ticket: int) -> None:
    """Block until the xc_correlate_host_async call `ticket` is complete."""
    check(lib().xc_host_wait(ctypes.c_uint64(ticket)))


class kernel_timing:
    """Context manager: CUDA-event time of the dense correlation kernels
    (plain and split-BF16) launched inside the block.  After exit,
    `total_ms` and `launches` hold the summed kernel time and the count."""

    def __enter__(self):
        check(lib().xc_kernel_timing(1))
        self.total_ms, self.launches = 0.0, 0
        return self

    def __exit__(self, *exc):
        ms, n = ctypes.c_double(), ctypes.c_uint32()
        try:
            check(lib().xc_kernel_timing_read(ctypes.byref(ms), ctypes.byref(n)))
        finally:
            lib().xc_kernel_timing(0)
        self.total_ms, self.launches = ms.value, n.value
        return False


class FftPlan:
    """Explicit FFT plan (xc_fft_plan_create); owns its cuFFT plans."""

    def __init__(self, mode, dtype, left_shape, n_left, right_shape, n_right, pad=(0, 0)):
        self.handle = ctypes.c_void_p()
        check(lib().xc_fft_plan_create(ctypes.byref(self.handle), MODES[mode], DTYPES[dtype], size2(*left_shape),
                                       n_left, size2(*right_shape), n_right, size2(*pad)))
        b = ctypes.c_size_t()
        check(lib().xc_fft_plan_workspace_size(self.handle, ctypes.byref(b)))
        self.workspace_bytes = int(b.value)
        p = Size2()
        check(lib().xc_fft_plan_pad_size(self.handle, ctypes.byref(p)))
        self.pad = (int(p.y), int(p.x))

    def execute(self, left, right, out, workspace, normalize=True, stream=None):
        check(lib().xc_fft_execute(self.handle, left.data_ptr(), right.data_ptr(), out.data_ptr(), int(normalize),
                                   workspace.data_ptr(), workspace.numel(), _stream_ptr(stream)))
        return out

    def close(self):
        if self.handle:
            lib().xc_fft_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Ragged batches
# ---------------------------------------------------------------------------
def pack(mats, dtype=np.float32):
    """Stack matrices of any sizes into one flat array + MatrixDesc array."""
    descs = (MatrixDesc * len(mats))()
    off = 0
    for i, m in enumerate(mats):
        descs[i] = MatrixDesc(off, m.shape[0], m.shape[1])
        off += m.size
    flat = np.concatenate([np.ascontiguousarray(m, dtype=dtype).ravel() for m in mats]) if mats else \
        np.zeros(0, dtype)
    return flat, descs


def pair_layout(lefts, rights, pairs):
    """PairDesc array and total output elements for (left, right) index pairs."""
    pd = (PairDesc * len(pairs))()
    off = 0
    shapes = []
    for i, (a, b) in enumerate(pairs):
        sy = lefts[a].shape[0] + rights[b].shape[0] - 1
        sx = lefts[a].shape[1] + rights[b].shape[1] - 1
        pd[i] = PairDesc(a, b, off)
        shapes.append((off, sy, sx))
        off += sy * sx
    return pd, off, shapes


class RaggedPlan:
    """A ragged batch bound to device buffers (xc_ragged_plan_create)."""

    def __init__(self, lefts, rights, pairs, dtype="f32"):
        import torch

        npdt = np.float32 if dtype == "f32" else np.float64
        tdt = torch.float32 if dtype == "f32" else torch.float64
        lflat, self.ldesc = pack(lefts, npdt)
        rflat, self.rdesc = pack(rights, npdt)
        self.pdesc, n_out, self.shapes = pair_layout(lefts, rights, pairs)
        self.left = torch.from_numpy(lflat).cuda()
        self.right = torch.from_numpy(rflat).cuda()
        self.out = torch.zeros(n_out, dtype=tdt, device="cuda")
        self.dtype = dtype
        self.handle = ctypes.c_void_p()
        check(lib().xc_ragged_plan_create(ctypes.byref(self.handle), DTYPES[dtype], self.left.data_ptr(), self.ldesc,
                                          len(lefts), self.right.data_ptr(), self.rdesc, len(rights), self.pdesc,
                                          len(pairs), self.out.data_ptr()))

    def autotune(self, stream=None):
        """Times the plan's variants; returns (chosen variant, its ms per
        step, or < 0 when the choice came from the cache)."""
        variant = ctypes.c_int()
        ms = ctypes.c_double()
        check(lib().xc_ragged_autotune(self.handle, _stream_ptr(stream), ctypes.byref(variant), ctypes.byref(ms)))
        return variant.value, ms.value

    def describe(self, variant=-1):
        """Variant `variant` (-1: the chosen one) as a dict: its index, the
        plan's variant count, the plain kernel's tile shape, and the pairs run
        on the split-BF16 path (count and multiply-add threshold)."""
        v = RaggedVariant()
        check(lib().xc_ragged_describe(self.handle, variant, ctypes.byref(v)))
        return {"index": v.index, "n_variants": v.n_variants, "tile_shape": v.tile_shape, "tc_pairs": v.tc_pairs,
                "tc_min_macs": v.tc_min_macs}

    def select(self, variant):
        check(lib().xc_ragged_select(self.handle, variant))

    def execute(self, stream=None):
        check(lib().xc_ragged_execute(self.handle, _stream_ptr(stream)))

    def per_pair(self, out, stream=None):
        """The baseline: one plain-kernel launch per pair into `out`."""
        check(lib().xc_correlate_pairs(DTYPES[self.dtype], self.left.data_ptr(), self.ldesc, len(self.ldesc),
                                       self.right.data_ptr(), self.rdesc, len(self.rdesc), self.pdesc,
                                       len(self.pdesc), out.data_ptr(), _stream_ptr(stream)))

    def per_pair_streams(self, out, n_streams=8):
        """The reference's multi-stream driver (src/n_to_m.hpp:198-212): pair i
        goes to stream i % n_streams, one plain-kernel launch each; the
        current stream waits for all of them."""
        import torch

        if not hasattr(self, "_streams") or len(self._streams) != n_streams:
            self._streams = [torch.cuda.Stream() for _ in range(n_streams)]
            self._subsets = []
            for s in range(n_streams):
                sub = list(self.pdesc)[s::n_streams]
                self._subsets.append((PairDesc * len(sub))(*sub))
        cur = torch.cuda.current_stream()
        start = torch.cuda.Event()
        start.record(cur)
        for st, sub in zip(self._streams, self._subsets):
            st.wait_event(start)
            if len(sub):
                check(lib().xc_correlate_pairs(DTYPES[self.dtype], self.left.data_ptr(), self.ldesc, len(self.ldesc),
                                               self.right.data_ptr(), self.rdesc, len(self.rdesc), sub, len(sub),
                                               out.data_ptr(), st.cuda_stream))
        for st in self._streams:
            cur.wait_stream(st)

    def outputs(self, flat=None):
        flat = self.out if flat is None else flat
        host = flat.cpu().numpy()
        return [host[o:o + sy * sx].reshape(sy, sx) for o, sy, sx in self.shapes]

    def close(self):
        if self.handle:
            lib().xc_ragged_plan_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
