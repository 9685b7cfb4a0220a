"""Train the method selector on a measured timing dataset and report its
regret against the exhaustive autotune on the held-out workloads.

Usage: python train.py TIMINGS.npz WEIGHTS.npz [--steps 3000] [--seed 0]
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("timings")
    ap.add_argument("weights")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--seed", type=int, default=0)
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
           "fft_2048x2048x16_choice": selector.METHOD_NAMES[int(chosen[-1])],
           "n_train": int(len(tr)), "n_heldout": int(len(te))}
    np.savez(args.weights, params=params, t_mean=mu, t_std=sd, steps=args.steps, seed=args.seed)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
