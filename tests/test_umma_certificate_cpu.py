"""The certificate of the batched kernel's tcgen05 path (ckm_umma_batch.cuh),
checked on the CPU by emulation.

The kernel splits every coordinate into fp16 halves (x = x_h + x_l), sums
x_h.c_l, x_l.c_h and then x_h.c_h in f32, forms the score
s = fma(-2, dot, |c|^2) in FP32 and calls a point proved when the two lowest
scores differ by more than T = A_D r^2 + B_D r + C_D (r = |x| + max|c|).
Here the same steps run in numpy, with several orders of the f32
accumulation.  Two checks:
  * the score error stays within half of T minus the reference's own
    distance error (the part of T the scores may use);
  * whenever the emulated screen certifies a label, it is the label of the
    reference's FP32 distance (t = x - c, fma(t, t, acc), strict '<',
    kmeans_naive.cpp:48-63), on sets with many near ties.
"""
import numpy as np
import pytest

U = 2.0 ** -24


def bound_constants(D):
    """A_D, B_D, C_D as in UmmaBound<D> (float32 arithmetic there; float64 here)."""
    gamma = 2.0 * D * 2.0 ** -23 * 1.005
    A = (3.001 * 2.0 ** -22 + 1.01 * gamma + 5.2 * 2.0 ** -24 + 2.0 * (D + 4) * 2.0 ** -24) * 1.001
    B = 4.1 * 2.0 ** -25 * (8.0 if D == 64 else 6.0) * 1.001
    C = 2.0 ** -40
    return A, B, C


def split16(v):
    v = np.asarray(v, np.float32)
    h = v.astype(np.float16)
    lo = (v - h.astype(np.float32)).astype(np.float16)
    return h.astype(np.float32), lo.astype(np.float32)


def f32_sum(terms, order):
    """Sum of the rows of `terms` (shape [K, ...]) in float32, one rounding per
    addition, in the given order of the K terms."""
    acc = np.zeros(terms.shape[1:], np.float32)
    for i in order:
        acc = (acc + terms[i].astype(np.float32)).astype(np.float32)
    return acc


def emulated_scores(X, C, order_kind, rng):
    """Scores [n, k] as the kernel forms them (cross products first)."""
    n, D = X.shape
    xh, xl = split16(X)
    ch, cl = split16(C)
    # products are exact in float32 (11 x 11 significant bits)
    cross = np.concatenate([(xh[:, None, :] * cl[None, :, :]), (xl[:, None, :] * ch[None, :, :])], axis=2)
    main = xh[:, None, :] * ch[None, :, :]
    cross = np.moveaxis(cross.astype(np.float32), 2, 0)
    main = np.moveaxis(main.astype(np.float32), 2, 0)
    if order_kind == "sequential":
        oc, om = np.arange(cross.shape[0]), np.arange(D)
    elif order_kind == "reversed":
        oc, om = np.arange(cross.shape[0])[::-1], np.arange(D)[::-1]
    else:
        oc, om = rng.permutation(cross.shape[0]), rng.permutation(D)
    acc = f32_sum(cross, oc)
    for i in om:
        acc = (acc + main[i]).astype(np.float32)
    cn = (C.astype(np.float64) ** 2).sum(1).astype(np.float32)
    s = (-2.0 * acc.astype(np.float64) + cn[None, :].astype(np.float64)).astype(np.float32)
    return s


def reference_distances(X, C):
    """The reference's FP32 distance: t = x - c, acc = fma(t, t, acc), f ascending."""
    n, D = X.shape
    acc = np.zeros((n, C.shape[0]), np.float32)
    for f in range(D):
        t = (X[:, None, f] - C[None, :, f]).astype(np.float32)
        acc = (t.astype(np.float64) * t + acc).astype(np.float32)  # one rounding, as fma
    return acc


def reference_labels(dist):
    best = np.full(dist.shape[0], np.finfo(np.float32).max, np.float32)
    lab = np.zeros(dist.shape[0], np.int64)
    for c in range(dist.shape[1]):
        lt = dist[:, c] < best
        best = np.where(lt, dist[:, c], best)
        lab = np.where(lt, c, lab)
    return lab


def near_tie_set(rng, n, D, k, spread):
    """Points around centres, a third of which have an almost duplicated
    twin; one exact duplicate (centroids 0 and 1) and a few points midway
    between two centroids."""
    centres = rng.uniform(-10, 10, (k - k // 4, D))
    twins = centres[: k // 4] + rng.normal(0, spread, (k // 4, D))
    C = np.concatenate([centres, twins]).astype(np.float32)
    C[1] = C[0]  # an exact tie
    X = (C[rng.integers(0, k, n)] + rng.normal(0, 1.0, (n, D))).astype(np.float32)
    X[:8] = (C[0] + C[2]) / 2  # equidistant points
    return X, C


@pytest.mark.parametrize("D", [32, 64])
@pytest.mark.parametrize("order_kind", ["sequential", "reversed", "shuffled"])
def test_score_error_within_the_bound(D, order_kind):
    rng = np.random.default_rng(D + len(order_kind))
    A, B, Cc = bound_constants(D)
    for scale in (1e-3, 1.0, 40.0, 3000.0):
        X = (rng.normal(0, 1, (300, D)) * scale).astype(np.float32)
        C = (rng.normal(0, 1, (40, D)) * scale).astype(np.float32)
        X[:5, : D // 2] = 0.0
        X[5:10] *= np.float32(2.0 ** -20)  # fp16 subnormal range
        s = emulated_scores(X, C, order_kind, rng).astype(np.float64)
        Xd, Cd = X.astype(np.float64), C.astype(np.float64)
        exact = (Cd ** 2).sum(1)[None, :] - 2.0 * Xd @ Cd.T
        a = np.sqrt((Xd ** 2).sum(1))
        cm = np.sqrt((Cd ** 2).sum(1)).max()
        r = a + cm
        T = A * r * r + B * r + Cc
        # T = 2 (score error bound) + 2 (D + 4) u r^2: the scores may use half
        # of what is left after the reference's own error
        score_budget = (T - 2.0 * (D + 4) * U * r * r) / 2.0
        err = np.abs(s - exact).max(1)
        assert np.all(err <= score_budget), (scale, float((err / score_budget).max()))


@pytest.mark.parametrize("D", [32, 64])
@pytest.mark.parametrize("spread", [1e-4, 1e-2, 0.3])
def test_certified_labels_are_the_reference_labels(D, spread):
    rng = np.random.default_rng(int(D * 1000 + spread * 1e4))
    A, B, Cc = bound_constants(D)
    n, k = 1500, 24
    X, C = near_tie_set(rng, n, D, k, spread)
    ref = reference_labels(reference_distances(X, C))
    for order_kind in ("sequential", "shuffled"):
        s = emulated_scores(X, C, order_kind, rng)
        order = np.argsort(s, axis=1, kind="stable")
        m1 = s[np.arange(n), order[:, 0]].astype(np.float64)
        m2 = s[np.arange(n), order[:, 1]].astype(np.float64)
        i1 = order[:, 0]
        a = np.sqrt((X.astype(np.float64) ** 2).sum(1)) * (1 + 2.0 ** -16)
        cm = np.sqrt((C.astype(np.float64) ** 2).sum(1)).max()
        r = (a + cm) * (1 + 2.0 ** -20)
        T = A * r * r + B * r + Cc
        proved = (m2 - m1) > T
        assert np.all(i1[proved] == ref[proved]), int((i1[proved] != ref[proved]).sum())
        # a point whose nearest centroid is the duplicated pair 0 / 1 has two
        # equal lowest scores: never proved
        assert not np.any(proved[ref == 0])
        assert np.any(ref == 0)
        assert proved.mean() > 0.2


def _header_constants(D):
    """UmmaBound<D>'s constants, evaluated from the header's own expressions."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "cl-kmeans_gb300", "csrc", "ckm_umma_batch.cuh")).read()
    body = re.search(r"struct UmmaBound \{(.*?)\n\};", src, re.S).group(1)
    env = {"D": D}
    for name in ("gamma", "A", "B", "C"):
        expr = re.search(r"static constexpr float %s\s*=\s*(.*?);" % name, body, re.S).group(1)
        expr = re.sub(r"0x1p(-?\d+)f", r"(2.0 ** \1)", expr)
        expr = re.sub(r"(\d+\.\d+)f", r"\1", expr).replace("(float)", "")
        expr = re.sub(r"\(D == 64 \? ([\d.]+) : ([\d.]+)\)", r"(\1 if D == 64 else \2)", expr)
        env[name] = eval(expr, {}, env)
    return env["A"], env["B"], env["C"]


@pytest.mark.parametrize("D", [32, 64])
def test_emulated_bound_is_the_kernels(D):
    """The constants checked above are the ones the kernel uses."""
    got = _header_constants(D)
    for a, b in zip(got, bound_constants(D)):
        assert a == pytest.approx(b, rel=1e-6)
