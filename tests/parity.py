"""End-to-end parity helpers: FP64 adjudication of label mismatches against a
derived bound, and centroid error against an FP64 oracle.

Two runs of Lloyd's iteration (ours and the oracle's restatement of the
reference's KmeansNaive, kmeans_naive.cpp:48-100) start from the same
centroids and use the same FP32 distance arithmetic, so in any iteration where
both see the same input centroids their labels are bit-identical (the
lockstep tests check that).  Their centroids still differ by rounding: our
per-CTA FP32 partial sums merge in FP64, the reference sums in FP32 with Kahan
compensation (kmeans_naive.cpp:70-94).  After several iterations a point can
therefore sit on different sides of a near tie in the two runs.  Such a point
is accepted only if this bound, derived from the FP32 rounding of a distance
and the measured centroid drift, explains it:

  rho = (d + 4) * 2^-24   relative error of the reference's FP32 distance
                          (t = x - c rounded, fma(t, t, acc) chained over d
                          features; the same rho the kernels' certificates use)
  f   = sqrt((1 + rho) / (1 - rho))

With a = our label, b = the oracle's, Cg / Cr the two runs' input centroids of
the last iteration, delta_c = |Cg_c - Cr_c|_2 and D(x, c) exact squared
distances, our FP32 choice of a implies D(x, Cg_a) <= (1+rho)/(1-rho) D(x, Cg_b),
and the triangle inequality moves both sides to the oracle's centroids:

  sqrt(D(x, Cr_a)) - sqrt(D(x, Cr_b)) <= (f - 1) sqrt(D(x, Cr_b)) + f delta_b + delta_a.

Every mismatch is checked against this inequality in FP64; there is no cap on
their number and no ad-hoc gap threshold.  A mismatch outside it is a label
the FP32 arithmetic cannot produce, i.e. a bug.
"""
import numpy as np


def rho(d):
    return (d + 4) * 2.0 ** -24


def rows(C, d, k):
    """Column-major centroids C[f * k + c] -> (k, d) float64."""
    return np.asarray(C, np.float64).reshape(d, k).T


def adjudicate(P, n, d, k, L_ours, L_ref, C_ours_prev, C_ref_prev, prev_slack_ulps=0):
    """Adjudicate every label mismatch in FP64 (module docstring).  Returns a
    dict with the mismatch count, the largest gap / bound ratio and the
    largest centroid drift; raises AssertionError on a mismatch the bound
    does not explain.

    prev_slack_ulps: when C_ours_prev comes from a rerun of the same job on
    another path (a batched or served job rerun alone), the two paths' FP64
    merges of the same FP32 partial sums can round to FP32 one ulp apart; the
    drift then gets that many ulps per coordinate (of the centroid's largest
    coordinate) added."""
    L_ours = np.asarray(L_ours).astype(np.int64)
    L_ref = np.asarray(L_ref).astype(np.int64)
    mism = np.nonzero(L_ours != L_ref)[0]
    Cg, Cr = rows(C_ours_prev, d, k), rows(C_ref_prev, d, k)
    with np.errstate(invalid="ignore"):
        drift = np.sqrt(((Cg - Cr) ** 2).sum(axis=1))
        if prev_slack_ulps:
            drift += prev_slack_ulps * np.sqrt(d) * 2.0 ** -23 * np.abs(Cg).max(axis=1)
    finite = np.isfinite(drift)
    out = {"mismatches": int(mism.size), "worst_gap_over_bound": 0.0,
           "max_drift": float(drift[finite].max()) if finite.any() else 0.0}
    if mism.size == 0:
        return out
    X = np.asarray(P, np.float64).reshape(d, n)[:, mism].T          # (m, d)
    a, b = L_ours[mism], L_ref[mism]
    Dra = ((X - Cr[a]) ** 2).sum(axis=1)
    Drb = ((X - Cr[b]) ** 2).sum(axis=1)
    f = np.sqrt((1 + rho(d)) / (1 - rho(d)))
    gap = np.sqrt(Dra) - np.sqrt(Drb)
    bound = (f - 1) * np.sqrt(Drb) + f * drift[b] + drift[a] + 1e-30
    ratio = gap / bound
    out["worst_gap_over_bound"] = float(np.nanmax(ratio))
    bad = ~(gap <= bound)
    assert not bad.any(), ("%d of %d label mismatches are outside the derived near-tie bound "
                           "(first: point %d, ours %d, oracle %d, gap %.3g, bound %.3g)"
                           % (int(bad.sum()), mism.size, int(mism[bad][0]), int(a[bad][0]), int(b[bad][0]),
                              float(gap[bad][0]), float(bound[bad][0])))
    return out


def rel_centroid_error(C, C_ref):
    """Normwise relative centroid error max |C - C_ref| / max |C_ref| over the
    clusters non-empty in both (NaN = empty)."""
    C = np.asarray(C, np.float64)
    R = np.asarray(C_ref, np.float64)
    ok = np.isfinite(C) & np.isfinite(R)
    if not ok.any():
        return 0.0
    return float(np.abs(C[ok] - R[ok]).max() / max(np.abs(R[ok]).max(), 1e-300))
