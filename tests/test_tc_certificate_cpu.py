"""The certificate of the tensor-core labelling (ckm_tc.cu, tc_params_kernel
and tc_label_kernel), checked on the CPU by emulation.

The kernel scales points and centroids by powers of two (sx, sc) so that
every coordinate fits fp16, rounds them to fp16 once, accumulates the dot
products in f32 (the order inside the tensor core is not specified, so several
orders are emulated), forms the score s = fma(alpha, dot, |c|^2) with
alpha = -2 / (sx sc) and keeps as candidates every cluster whose score is
within T of the lowest, with
  T = (t2 (|x| + cm)^2 + te |e| + t1 |x| + t0) (1 + 2^-10),
  t1 = (4 fm + 4 g (cm + fm)) s,  te = (4 (cm + fm) + 4 g (cm + fm)) s,
  t2 = (2 2^-23 1.01 + 2 (d + 2) 2^-24 1.01) s,  t0 = (d + 8) 2^-146,
  s = 1 + 2^-10,  g = 2 d_pad 2^-23,
where |e| bounds the point's rounding error, fm the centroids' and
cm >= max |c|.  The check: on sets full of near ties and exact ties, the
label of the reference's FP32 distance (t = x - c, fma(t, t, acc), strict '<',
kmeans_naive.cpp:48-63) is always among the candidates, and a point with one
candidate gets exactly that label.
"""
import math

import numpy as np
import pytest


def scale_exponent(maxabs):
    """2^e maxabs <= 2^15, e in [-60, 60] (scale_exponent in ckm_tc.cu)."""
    if not (maxabs > 0) or math.isinf(maxabs):
        return 0
    _, e = math.frexp(maxabs)
    return max(-60, min(60, 15 - e))


def reference_labels(X, C):
    n, d = X.shape
    acc = np.zeros((n, C.shape[0]), np.float32)
    for f in range(d):
        t = (X[:, None, f] - C[None, :, f]).astype(np.float32)
        acc = (t.astype(np.float64) * t + acc).astype(np.float32)  # one rounding, as fma
    best = np.full(n, np.finfo(np.float32).max, np.float32)
    lab = np.zeros(n, np.int64)
    for c in range(C.shape[0]):
        better = acc[:, c] < best
        best = np.where(better, acc[:, c], best)
        lab = np.where(better, c, lab)
    return lab


def emulated_candidates(X, C, order_kind, rng):
    n, d = X.shape
    d_pad = (d + 63) // 64 * 64
    sx = 2.0 ** scale_exponent(float(np.abs(X).max()))
    sc = 2.0 ** scale_exponent(float(np.abs(C).max()))
    xq = (X.astype(np.float64) * sx).astype(np.float32).astype(np.float16).astype(np.float32)
    cq = (C.astype(np.float64) * sc).astype(np.float32).astype(np.float16).astype(np.float32)
    # fp16 x fp16 products are exact in f32; f32 accumulation in one of several orders
    order = {"sequential": np.arange(d), "reversed": np.arange(d)[::-1], "random": rng.permutation(d)}[order_kind]
    dot = np.zeros((n, C.shape[0]), np.float32)
    for f in order:
        dot = (dot + xq[:, None, f] * cq[None, :, f]).astype(np.float32)
    cn = (C.astype(np.float64) ** 2).sum(1).astype(np.float32)
    alpha = -2.0 / (sx * sc)
    s = (alpha * dot.astype(np.float64) + cn[None, :]).astype(np.float32)
    # the bounds the kernel forms (upper bounds of the exact quantities)
    xn = np.sqrt((X.astype(np.float64) ** 2).sum(1)) * (1 + 2.0 ** -14)
    xe = np.sqrt(((xq.astype(np.float64) / sx - X) ** 2).sum(1)) * (1 + 2.0 ** -14)
    fm = float(np.sqrt(((cq.astype(np.float64) / sc - C) ** 2).sum(1)).max()) * (1 + 2.0 ** -40)
    cm = float(np.sqrt((C.astype(np.float64) ** 2).sum(1)).max()) * (1 + 2.0 ** -40)
    g = 2.0 * d_pad * 2.0 ** -23
    safety = 1.0 + 2.0 ** -10
    t1 = (4 * fm + 4 * g * (cm + fm)) * safety
    te = (4 * (cm + fm) + 4 * g * (cm + fm)) * safety
    t2 = (2 * 2.0 ** -23 * 1.01 + 2 * (d + 2) * 2.0 ** -24 * 1.01) * safety
    t0 = (d + 8) * 2.0 ** -146
    T = (t2 * (xn + cm) ** 2 + te * xe + t1 * xn + t0) * (1 + 2.0 ** -10)
    m = s.min(1).astype(np.float64)
    return s.astype(np.float64) <= (m + T)[:, None]


def near_tie_set(n, d, k, rng, spread):
    """Centroids from a few blobs (several per blob: many near ties), two
    exact duplicates, and points on and around the bisectors of centroid
    pairs as well as around the centroids."""
    centres = rng.normal(0.0, spread, (max(2, k // 4), d))
    C = centres[rng.integers(0, len(centres), k)] + rng.normal(0.0, 0.3, (k, d))
    C[1] = C[0]                                # an exact tie: cluster 0 wins
    C = C.astype(np.float32)
    a = rng.integers(0, k, n)
    b = rng.integers(0, k, n)
    mid = 0.5 * (C[a].astype(np.float64) + C[b])
    X = np.where(rng.random((n, 1)) < 0.5, mid + rng.normal(0.0, 1e-3, (n, d)),
                 C[a] + rng.normal(0.0, 0.5, (n, d)))
    return X.astype(np.float32), C


@pytest.mark.parametrize("d,k,spread", [(128, 256, 2.0), (100, 64, 20.0), (64, 300, 0.05), (200, 40, 300.0)])
@pytest.mark.parametrize("order_kind", ["sequential", "reversed", "random"])
def test_reference_label_is_always_a_candidate(d, k, spread, order_kind):
    rng = np.random.default_rng(d * 1000 + k)
    X, C = near_tie_set(1500, d, k, rng, spread)
    ref = reference_labels(X, C)
    cand = emulated_candidates(X, C, order_kind, rng)
    missing = ~cand[np.arange(len(ref)), ref]
    assert not missing.any(), "%d points lose their reference label" % int(missing.sum())
    single = cand.sum(1) == 1
    assert np.array_equal(cand[single].argmax(1), ref[single])
    # the set does hold near ties: some points keep several candidates
    assert (cand.sum(1) >= 2).any()
