"""Train the method selector on a measured timing dataset and report its
regret against the exhaustive autotune on the held-out workloads.

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


def baselines(times, M, X):
    """Selectors without the network, for comparison."""
    out = {}
    for k, name in enumerate(selector.METHOD_NAMES):
        chosen = np.where(M[:, k] > 0, k, 0)  # fall back to direct where unsupported
        out[f"always_{name}"] = selector.regret(times, chosen)
    return out


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
    res = {"train_loss": hist, "heldout_regret_total": selector.regret(times[te], chosen)[0],
           "heldout_regret_mean": selector.regret(times[te], chosen)[1],
           "heldout_pick_accuracy": float(np.mean(chosen == times[te].argmin(axis=1))),
           "baselines_heldout": {k: v[0] for k, v in baselines(times[te], M[te], X[te]).items()},
           "exhaustive_autotune_cost_over_best": float(
               (np.where(M[te] > 0, times[te], 0).sum(axis=1) + times[te].min(axis=1)).sum()
               / times[te].min(axis=1).sum()),
           "fft_2048x2048x16_choice": selector.METHOD_NAMES[int(chosen[-1])],
           "n_train": int(len(tr)), "n_heldout": int(len(te))}
    np.savez(args.weights, params=params, t_mean=mu, t_std=sd, steps=args.steps, seed=args.seed)
    if args.inc:
        write_inc(args.inc, params, os.path.basename(args.timings), args.steps, args.seed)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
