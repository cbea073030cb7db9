"""Generates the golden fixtures in this directory from the reference's own
KmeansNaive (kmeans_naive.cpp), compiled unchanged by oracle/build_ref.sh.

Run here (where the reference tree exists):
    oracle/build_ref.sh && python tests/golden/make_golden.py

Each case stores its seeded inputs (column-major points, initial centroids)
and the reference's outputs after the stated iteration count.  The inputs are
made by numpy from the seed below, so the script is reproducible.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def blobs(n, d, kb, seed, spread=10.0, sigma=1.0):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-spread, spread, size=(kb, d))
    X = centres[rng.integers(0, kb, size=n)] + sigma * rng.standard_normal((n, d))
    return np.ascontiguousarray(X.astype(np.float32).T).reshape(-1)


def lattice(n, d, seed):
    """Integer lattice points: many exact distance ties."""
    rng = np.random.default_rng(seed)
    X = rng.integers(-3, 4, size=(n, d)).astype(np.float32)
    return np.ascontiguousarray(X.T).reshape(-1)


CASES = [
    # name, (n, d, k, iterations), points factory, type
    ("c1_small", (4096, 4, 10, 30), lambda: blobs(4096, 4, 10, 101), "f32"),
    ("ragged", (4099, 3, 7, 10), lambda: blobs(4099, 3, 7, 102), "f32"),
    ("empty_clusters", (50, 2, 60, 3), lambda: blobs(50, 2, 5, 103), "f32"),
    ("d1", (1000, 1, 5, 5), lambda: blobs(1000, 1, 5, 104), "f32"),
    ("d17", (333, 17, 9, 4), lambda: blobs(333, 17, 9, 105), "f32"),
    ("lattice_ties", (512, 2, 8, 6), lambda: lattice(512, 2, 106), "f32"),
    ("k1", (777, 4, 1, 2), lambda: blobs(777, 4, 3, 107), "f32"),
    ("wide_d64", (2000, 64, 20, 3), lambda: blobs(2000, 64, 20, 108), "f32"),
    ("f64_small", (2000, 3, 6, 8), lambda: blobs(2000, 3, 6, 109), "f64"),
]


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref not built: run oracle/build_ref.sh first")
    for name, (n, d, k, it), make, typ in CASES:
        P = make()
        if typ == "f32":
            C0 = O.first_x_f32(P, n, d, k)
            C, M, L = O.ref_naive_f32(P, n, d, k, it)
        else:
            P = P.astype(np.float64)
            C0 = O.first_x_f32(P.astype(np.float32), n, d, k).astype(np.float64)
            C, M, L = O.ref_naive_f64(P, n, d, k, it)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), points=P, centroids0=C0, centroids=C, masses=M,
                            labels=L, shape=np.array([n, d, k, it], np.int64), type=np.array(typ))
        print("wrote", name, "nan centroids:", int(np.isnan(C).sum()))


if __name__ == "__main__":
    main()
