"""Train the algorithm selector on a measured timing dataset and report its
regret against the exhaustive autotune (over the same candidates: method and
tile) on the held-out workloads, beside what selection without the network
costs: the best fixed candidate, and the exhaustive autotune that
XC_METHOD_AUTO runs on a problem's first call when no network is installed.

Usage: python train.py TIMINGS.npz WEIGHTS.npz [--inc selector_weights.inc]
                       [--steps 3000] [--seed 0]

--inc writes the trained parameters as a C array that the library compiles
in as the default network of XC_METHOD_AUTO (csrc/selector_weights.inc).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from xcorr import selector  # noqa: E402


FFT = selector.ALGO_NAMES.index("fft")  # supported by every problem


def baselines(times, M):
    """Fixed choices without the network (the FFT path where the fixed
    candidate does not support a problem), for comparison."""
    out = {}
    for k, name in enumerate(selector.ALGO_NAMES):
        chosen = np.where(M[:, k] > 0, k, FFT)
        out[f"always_{name}"] = selector.regret(times, chosen)
    return out


def default_tiles(timings_path):
    """Per workload, the candidate index each method runs with its default
    tile (tile 0): the plain kernel takes 8 partners per CTA (direct:1) when
    a left matrix has 4 or more partners, else one (direct:2); the split-BF16
    path takes items of 64 rows."""
    z = np.load(timings_path)
    idx = np.zeros((len(z["modes"]), 4), dtype=np.int64)
    for j, (m, b) in enumerate(zip(z["modes"], z["batch"])):
        n_l, n_r = selector.counts(str(m), int(b))
        partners = {"one_to_one": 1, "one_to_many": n_r, "n_to_mn": n_r // max(1, n_l), "n_to_m": n_r}[str(m)]
        idx[j] = [selector.ALGO_NAMES.index("direct:1" if partners >= 4 else "direct:2"),
                  selector.ALGO_NAMES.index("fft"), selector.ALGO_NAMES.index("tc_bf16x3:64"),
                  selector.ALGO_NAMES.index("tc_tf32x3")]
    return idx


def autotune_cost(times, M):
    """Total time of the exhaustive autotune's first call per problem: every
    supported candidate timed once, then the best run."""
    return float((np.where(M > 0, times, 0).sum(axis=1) + times.min(axis=1)).sum())


def write_inc(path, params, source, steps, seed):
    vals = ",\n".join(", ".join(f"{float(v):.9e}f" for v in params[i:i + 6]) for i in range(0, len(params), 6))
    with open(path, "w") as f:
        f.write(f"// Default weights of the method selector (XC_MLP_PARAMS floats in the layout of\n"
                f"// mlp.cu), trained by selector/train.py on {source}\n"
                f"// ({steps} full-batch Adam steps, seed {seed}).  Generated file.\n"
                f"#define XC_SELECTOR_BUILTIN 1\n"
                f"static const float kSelectorBuiltin[{len(params)}] = {{\n{vals}}};\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("timings")
    ap.add_argument("weights")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--inc", default=None)
    args = ap.parse_args()
    X, T, M, times = selector.load_dataset(args.timings)
    tr, te = selector.split(len(X), args.seed)
    Ts, mu, sd = selector.standardise(T[tr], M[tr])
    trainer = selector.Trainer(selector.init_params(args.seed))
    hist = trainer.fit(X[tr], Ts, M[tr], steps=args.steps)
    params = trainer.params()
    pred = selector.predict(params, X[te])
    chosen = selector.choose(pred, M[te])
    t = times[te]
    best = t.min(axis=1).sum()
    ours = t[np.arange(len(te)), chosen].sum()
    fixed = baselines(t, M[te])
    res = {"train_loss": hist, "heldout_regret_total": selector.regret(t, chosen)[0],
           "heldout_regret_mean": selector.regret(t, chosen)[1],
           "heldout_pick_accuracy": float(np.mean(chosen == t.argmin(axis=1))),
           "baselines_heldout": {k: v[0] for k, v in fixed.items()},
           "best_fixed": min(fixed, key=lambda k: fixed[k][0]),
           "network_over_best_fixed": float(ours / ((1 + min(v[0] for v in fixed.values())) * best)),
           "exhaustive_autotune_cost_over_best": autotune_cost(t, M[te]) / best,
           "fft_2048x2048x16_choice": selector.ALGO_NAMES[int(chosen[-1])],
           "n_train": int(len(tr)), "n_heldout": int(len(te))}
    # selection by method alone: the measured fastest method, each with its
    # default tile (what choosing the tile adds)
    dflt = default_tiles(args.timings)[te]
    by_method = dflt[np.arange(len(te)), np.argmin(np.take_along_axis(t, dflt, axis=1), axis=1)]
    z = np.load(args.timings)
    est = z["estimated"][te] if "estimated" in z else np.zeros_like(t, dtype=bool)
    res["method_only_oracle_regret_total"] = selector.regret(t, by_method)[0]
    res["fastest_candidate_counts_heldout"] = {n: int(np.sum(t.argmin(axis=1) == k))
                                               for k, n in enumerate(selector.ALGO_NAMES)}
    res["estimated_entries_heldout"] = int(est.sum())
    np.savez(args.weights, params=params, t_mean=mu, t_std=sd, steps=args.steps, seed=args.seed)
    if args.inc:
        write_inc(args.inc, params, os.path.basename(args.timings), args.steps, args.seed)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
