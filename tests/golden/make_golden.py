"""Regenerate the golden fixtures in this directory from the reference checkout.

Run once, where the reference source tree is available (it is read, never
modified):

    python tests/golden/make_golden.py /path/to/MK4H-cross-corr

It writes two kinds of fixtures:

1. ``data/*.csv.gz`` -- byte-for-byte gzip copies of the reference's shipped
   inputs and validated outputs (``data/ina_*.csv``, ``data/valid_*.csv``;
   naming explained in the reference's data/README.md).  These are the
   reference's own golden vectors.
2. ``scipy_cases.npz`` -- seeded random inputs and the outputs of the
   reference's Python implementation (``existing/python/crosscorr.py``:
   one_to_one / one_to_many / n_to_mn / n_to_m over scipy.signal.correlate2d,
   FP64), including odd sizes, 1xN strips and unequal left/right sizes that
   the reference CLI itself cannot load.

The tests never read the reference tree at run time; only these fixtures.
"""
from __future__ import annotations

import gzip
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (mode, n_left, n_right, (Hl, Wl), (Hr, Wr), seed, distribution)
CASES = [
    ("one_to_one", 1, 1, (17, 17), (17, 17), 11, "uniform"),
    ("one_to_one", 1, 1, (33, 20), (33, 20), 12, "normal"),
    ("one_to_one", 1, 1, (1, 45), (1, 45), 13, "uniform"),
    ("one_to_one", 1, 1, (40, 1), (40, 1), 14, "normal"),
    ("one_to_one", 1, 1, (23, 37), (9, 14), 15, "normal"),
    ("one_to_one", 1, 1, (5, 6), (19, 31), 16, "uniform"),
    ("one_to_many", 1, 3, (31, 31), (31, 31), 21, "uniform"),
    ("one_to_many", 1, 5, (16, 48), (7, 9), 22, "normal"),
    ("n_to_mn", 2, 6, (19, 19), (19, 19), 31, "normal"),
    ("n_to_mn", 3, 3, (12, 29), (12, 29), 32, "uniform"),
    ("n_to_m", 3, 4, (21, 21), (21, 21), 41, "normal"),
    ("n_to_m", 2, 3, (10, 34), (25, 8), 42, "uniform"),
]


def _gen(rng, shape, dist):
    if dist == "uniform":
        return rng.random(shape)
    return rng.standard_normal(shape)


def main(ref_root: str) -> None:
    data_src = os.path.join(ref_root, "data")
    data_dst = os.path.join(HERE, "data")
    os.makedirs(data_dst, exist_ok=True)
    for name in sorted(os.listdir(data_src)):
        if not name.endswith(".csv"):
            continue
        with open(os.path.join(data_src, name), "rb") as fi, \
                gzip.GzipFile(os.path.join(data_dst, name + ".gz"), "wb", 9, mtime=0) as fo:
            shutil.copyfileobj(fi, fo)

    sys.path.insert(0, os.path.join(ref_root, "existing", "python"))
    import crosscorr  # noqa: E402  (the reference's SciPy implementation)
    from matrix import MatrixArray  # noqa: E402

    arrays = {}
    for idx, (mode, n, m, ls, rs, seed, dist) in enumerate(CASES):
        rng = np.random.default_rng(seed)
        left = _gen(rng, (n,) + ls, dist).astype(np.float32).astype(np.float64)
        right = _gen(rng, (m,) + rs, dist).astype(np.float32).astype(np.float64)
        la = MatrixArray(ls, n, left.reshape(n * ls[0], ls[1]))
        ra = MatrixArray(rs, m, right.reshape(m * rs[0], rs[1]))
        res = getattr(crosscorr, mode)(la, ra)
        out = np.asarray(res.data).reshape(res.num_matrices, res.matrix_size[0], res.matrix_size[1])
        arrays[f"c{idx}_left"] = left
        arrays[f"c{idx}_right"] = right
        arrays[f"c{idx}_out"] = out
        arrays[f"c{idx}_mode"] = np.array(mode)
    np.savez_compressed(os.path.join(HERE, "scipy_cases.npz"), **arrays)
    print(f"wrote {len(CASES)} scipy cases and the reference data files")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
