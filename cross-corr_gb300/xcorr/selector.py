"""The learned algorithm selector: data, training on the GPU with the
library's own MLP kernels (xc_mlp_gradient / xc_mlp_adam_step), evaluation
against the exhaustive autotune, and installation for XC_METHOD_AUTO.

The network predicts the standardised log run time of each candidate
algorithm -- a method and one of its tiles (xc_algorithm): the plain kernel's
three tile shapes, the FFT path, split-BF16 with items of at most 32 or 64
left rows, split-TF32 -- from 8 features (xc_selector_features); the selector
picks the smallest prediction among the candidates a problem supports.  Its
regret is measured against the exhaustive autotune over the same candidates
(the measured fastest) on held-out workloads.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import DTYPES, METHODS, MODES, Algo, check, lib, size2

# the candidates in the order of the network's outputs (xc_algorithm)
ALGO_NAMES = ["direct:1", "direct:2", "direct:3", "fft", "tc_bf16x3:32", "tc_bf16x3:64", "tc_tf32x3"]
N_OUT = len(ALGO_NAMES)
N_PARAMS = 64 * 8 + 64 + 64 * 64 + 64 + N_OUT * 64 + N_OUT


def algo_struct(name):
    """'method' or 'method:tile' -> xc_algo."""
    method, _, tile = name.partition(":")
    return Algo(METHODS[method], int(tile) if tile else 0)


def algo_name(a):
    method = {v: k for k, v in METHODS.items()}[a.method]
    if method in ("auto", "fft", "tc_tf32x3") or a.tile == 0:
        return method
    return f"{method}:{a.tile}"


def counts(mode, batch):
    """Left/right matrix counts of a workload of `batch` outputs (the dataset's convention)."""
    if mode == "one_to_one":
        return 1, 1
    if mode == "one_to_many":
        return 1, batch
    if mode == "n_to_mn":
        return 2, 2 * math.ceil(batch / 2)
    return 2, math.ceil(batch / 2)


def features(mode, left_shape, n_left, right_shape, n_right):
    f = (ctypes.c_float * 8)()
    check(lib().xc_selector_features(MODES[mode], size2(*left_shape), n_left, size2(*right_shape), n_right, f))
    return np.array(f[:], dtype=np.float32)


def load_dataset(path):
    """Features X (n,8), log10 times T (n,7) with inf for unsupported, mask M."""
    z = np.load(path)
    modes = [str(m) for m in z["modes"]]
    rows = []
    for m, sl, sr, b in zip(modes, z["sides_left"], z["sides_right"], z["batch"]):
        n_left, n_right = counts(m, int(b))
        rows.append(features(m, (int(sl), int(sl)), n_left, (int(sr), int(sr)), n_right))
    X = np.stack(rows)
    times = np.asarray(z["times"], dtype=np.float64)
    M = np.isfinite(times).astype(np.float32)
    T = np.where(M > 0, np.log10(np.where(M > 0, times, 1.0)), 0.0)
    return X, T, M, times


def split(n_workloads, seed=0, n_train=3072):
    """Seeded split of the 4096 sweep workloads into training and held-out sets;
    the dataset's final entry (the 2048x2048 one_to_many FFT case) is held out too."""
    perm = np.random.default_rng(seed).permutation(n_workloads - 1)
    return perm[:n_train], np.concatenate([perm[n_train:], [n_workloads - 1]])


def init_params(seed=0):
    """He-normal weights, zero biases."""
    rng = np.random.default_rng(seed)
    parts = []
    for shape in [(64, 8), (64,), (64, 64), (64,), (N_OUT, 64), (N_OUT,)]:
        parts.append(rng.standard_normal(shape) * math.sqrt(2.0 / shape[1]) if len(shape) == 2 else np.zeros(shape))
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


class Trainer:
    """Full-batch Adam on the GPU with the library's kernels."""

    def __init__(self, params):
        import torch
        self.torch = torch
        self.p = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).cuda()
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.g = torch.zeros_like(self.p)
        self.loss = torch.zeros(1, device="cuda")
        self.t = 0

    def gradient(self, X, T, M):
        """One masked-MSE gradient on device tensors; returns (grad, loss)."""
        check(lib().xc_mlp_gradient(self.p.data_ptr(), X.data_ptr(), T.data_ptr(), M.data_ptr(), X.shape[0],
                                    float(M.sum().item()), self.g.data_ptr(), self.loss.data_ptr(),
                                    self.torch.cuda.current_stream().cuda_stream))
        return self.g, self.loss

    def fit(self, X, T, M, steps=3000, lr=3e-3):
        torch = self.torch
        X = torch.as_tensor(X, dtype=torch.float32).cuda().contiguous()
        T = torch.as_tensor(T, dtype=torch.float32).cuda().contiguous()
        M = torch.as_tensor(M, dtype=torch.float32).cuda().contiguous()
        count = float(M.sum().item())
        L = lib()
        st = torch.cuda.current_stream().cuda_stream
        history = []
        for k in range(steps):
            check(L.xc_mlp_gradient(self.p.data_ptr(), X.data_ptr(), T.data_ptr(), M.data_ptr(), X.shape[0],
                                    count, self.g.data_ptr(), self.loss.data_ptr(), st))
            self.t += 1
            # cosine decay of the learning rate
            lr_k = lr * 0.5 * (1 + math.cos(math.pi * k / steps))
            check(L.xc_mlp_adam_step(self.p.data_ptr(), self.g.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                     self.t, lr_k, st))
            if k % 500 == 0 or k == steps - 1:
                history.append(float(self.loss.item()))
        return history

    def params(self):
        return self.p.cpu().numpy()


def predict(params, X):
    """Batched inference with xc_mlp_forward."""
    import torch
    p = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).cuda()
    x = torch.as_tensor(X, dtype=torch.float32).cuda().contiguous()
    y = torch.empty((x.shape[0], N_OUT), device="cuda")
    check(lib().xc_mlp_forward(p.data_ptr(), x.data_ptr(), x.shape[0], y.data_ptr(),
                               torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return y.cpu().numpy()


def choose(pred, M):
    """Index of the smallest prediction among supported methods."""
    return np.where(M > 0, pred, np.inf).argmin(axis=1)


def regret(times, chosen):
    """Aggregate regret: total time of the chosen methods over the total time
    of the measured fastest ones, minus one; also the mean per-workload ratio."""
    best = times.min(axis=1)
    got = times[np.arange(len(chosen)), chosen]
    return float(got.sum() / best.sum() - 1.0), float(np.mean(got / best) - 1.0)


def standardise(T, M):
    mu = float((T * M).sum() / M.sum())
    sd = float(np.sqrt(((T - mu) ** 2 * M).sum() / M.sum()))
    return (T - mu) / sd, mu, sd


def install(params):
    """Make XC_METHOD_AUTO use these weights (None uninstalls any network,
    "builtin" reinstalls the network compiled into the library)."""
    if isinstance(params, str) and params == "builtin":
        check(lib().xc_selector_load_builtin())
    elif params is None:
        check(lib().xc_selector_load(None))
    else:
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(lib().xc_selector_load(p.ctypes.data))


def select(mode, dtype, left_shape, n_left, right_shape, n_right):
    """The candidate XC_METHOD_AUTO runs ('auto' when neither a network nor a
    tuning record decides: the first correlation then autotunes)."""
    a = Algo()
    check(lib().xc_select_algorithm(MODES[mode], DTYPES[dtype], size2(*left_shape), n_left, size2(*right_shape),
                                    n_right, ctypes.byref(a)))
    return algo_name(a)


def autotune(mode, left, right, out, stream=None):
    """Exhaustive autotune (xc_autotune_algorithm) on device tensors: returns
    the fastest candidate's name and its time in ms."""
    import torch
    n_l, hl, wl = left.shape
    n_r, hr, wr = right.shape
    dtype = "f32" if left.dtype == torch.float32 else "f64"
    a = Algo()
    ms = ctypes.c_double()
    st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
    check(lib().xc_autotune_algorithm(MODES[mode], DTYPES[dtype], left.data_ptr(), size2(hl, wl), n_l,
                                      right.data_ptr(), size2(hr, wr), n_r, out.data_ptr(), st, ctypes.byref(a),
                                      ctypes.byref(ms)))
    return algo_name(a), ms.value


def time_algo(mode, left, right, out, name, reps=5):
    """Mean time (ms) of one correlation with candidate `name`, measured in
    the library (xc_time_algorithm: a warm-up call, then `reps` calls between
    CUDA events); the workspace is allocated outside the timed calls."""
    import torch
    from . import workspace_size
    n_l, hl, wl = left.shape
    n_r, hr, wr = right.shape
    dtype = "f32" if left.dtype == torch.float32 else "f64"
    a = algo_struct(name)
    method = {v: k for k, v in METHODS.items()}[a.method]
    wb = workspace_size(mode, dtype, method, (hl, wl), n_l, (hr, wr), n_r)
    ws = torch.empty(max(wb, 1), dtype=torch.uint8, device=left.device)
    ms = ctypes.c_double()
    check(lib().xc_time_algorithm(MODES[mode], DTYPES[dtype], a, left.data_ptr(), size2(hl, wl), n_l,
                                  right.data_ptr(), size2(hr, wr), n_r, out.data_ptr(), ws.data_ptr(), wb, reps,
                                  torch.cuda.current_stream().cuda_stream, ctypes.byref(ms)))
    return ms.value
