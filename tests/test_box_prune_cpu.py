"""Per-warp box pruning of the spatially ordered fused kernel (ckm_lowd.cu,
box_prune_mask), checked on the CPU: the kernel drops cluster c for a warp
when LB_c (1 - (D + 4) 2^-24) > min_c' UB_c' (1 + (D + 4) 2^-24) + 2^-120,
where LB_c / UB_c are the squared distances from c to the nearest / farthest
corner of the warp's bounding box, summed with downward / upward rounding.
Here those bounds are computed with exact rational arithmetic and exact
directed rounding to FP32, and every pruned cluster is checked to be
strictly farther, in the reference's FP32 distance (t = x - c,
fma(t, t, acc), kmeans_naive.cpp:52-57), than some kept cluster for every
point of the warp, so the reference's label is never pruned."""
from fractions import Fraction

import numpy as np
import pytest


def _round(q, up):
    """Directed rounding of the rational q to FP32."""
    v = np.float32(float(q))
    fv = Fraction(float(v))
    if up and fv < q:
        v = np.nextafter(v, np.float32(np.inf))
    elif not up and fv > q:
        v = np.nextafter(v, np.float32(-np.inf))
    return np.float32(v)


def sub(a, b, up):
    return _round(Fraction(float(a)) - Fraction(float(b)), up)


def fma_dir(a, b, c, up):
    return _round(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)), up)


def mul_dir(a, b, up):
    return _round(Fraction(float(a)) * Fraction(float(b)), up)


def prune_mask(P, C):
    """The kernel's decision per cluster (True = kept)."""
    D = P.shape[1]
    lo, hi = P.min(0), P.max(0)
    lbs, ubs = [], []
    for c in C:
        lb = np.float32(0.0)
        ub = np.float32(0.0)
        for f in range(D):
            g = max(sub(lo[f], c[f], False), sub(c[f], hi[f], False), np.float32(0.0))
            lb = fma_dir(g, g, lb, False)
            u = max(sub(c[f], lo[f], True), sub(lo[f], c[f], True), sub(c[f], hi[f], True), sub(hi[f], c[f], True))
            ub = fma_dir(u, u, ub, True)
        lbs.append(lb)
        ubs.append(ub)
    ub_min = min(ubs)
    k_lo = np.float32(1.0 - (D + 4) * 2.0 ** -24)
    k_hi = np.float32(1.0 + ((D + 5) // 2) * 2.0 ** -23)
    rhs = _round(Fraction(float(mul_dir(ub_min, k_hi, True))) + Fraction(2) ** -120, True)
    return np.array([not (mul_dir(lb, k_lo, False) > rhs) for lb in lbs])


def ref_dist(x, c):
    acc = np.float32(0.0)
    for f in range(len(x)):
        t = np.float32(x[f] - c[f])
        acc = np.float32(np.float64(t) * np.float64(t) + np.float64(acc))
    return acc


@pytest.mark.parametrize("D", [2, 4, 8])
@pytest.mark.parametrize("spread", [0.05, 1.0])
def test_pruned_clusters_are_never_the_reference_label(D, spread):
    rng = np.random.default_rng(D * 100 + int(spread * 10))
    pruned_total = 0
    for trial in range(12):
        C = rng.uniform(-10, 10, (16, D)).astype(np.float32)
        C[1] = C[0]                                            # an exact duplicate
        C[2] = C[0] + np.float32(1e-6)                         # a near duplicate
        centre = C[rng.integers(0, 16)] + rng.normal(0, 0.5, D)
        P = (centre + rng.normal(0, spread, (32, D))).astype(np.float32)
        P[0] = P.min(0)                                        # box corners are points
        P[1] = P.max(0)
        keep = prune_mask(P, C)
        assert keep.any()
        pruned_total += int((~keep).sum())
        for x in P:
            d = np.array([ref_dist(x, c) for c in C])
            best_kept = d[keep].min()
            # every pruned cluster is strictly farther than the best kept one
            assert np.all(d[~keep] > best_kept)
    assert pruned_total > 0  # the check is not vacuous


@pytest.mark.parametrize("D", [2, 4, 8])
def test_pruning_at_its_margin(D):
    """A warp whose points all coincide (the box is a point, LB = UB up to
    rounding) and a second cluster whose squared distance exceeds the first's
    by a relative delta swept across the pruning margin (about 2 (D + 4)
    2^-24): whenever the second cluster is pruned, the reference's distance
    to it is strictly larger."""
    rng = np.random.default_rng(D)
    pruned = kept = 0
    for trial in range(300):
        x = rng.uniform(-3, 3, D).astype(np.float32)
        u = rng.normal(0, 1, D)
        u /= np.linalg.norm(u)
        r0 = rng.uniform(0.5, 4.0)
        delta = rng.uniform(0.0, 8.0) * (D + 4) * 2.0 ** -24
        c0 = (x + u * r0).astype(np.float32)
        v = rng.normal(0, 1, D)
        v /= np.linalg.norm(v)
        c1 = (x + v * r0 * np.sqrt(1.0 + delta)).astype(np.float32)
        P = np.repeat(x[None, :], 32, axis=0)
        keep = prune_mask(P, np.stack([c0, c1]))
        d0, d1 = ref_dist(x, c0), ref_dist(x, c1)
        if not keep[1]:
            pruned += 1
            assert d1 > d0
        else:
            kept += 1
        if not keep[0]:
            assert d0 > d1
    assert pruned > 20 and kept > 20  # both sides of the margin were exercised
