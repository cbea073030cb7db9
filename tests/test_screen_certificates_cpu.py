"""The certified screens in front of the exact labelling, checked on the CPU
by emulation: their computed scores s_c = |c|^2 - 2 x.c stay within the
score part of the threshold T that the kernels use, so a point they call
proved has the reference's label.

  * FP32 screen (ckm_device.cuh, label_rows_screened): the dot product runs
    as two fma chains (even and odd features), added, then
    s = fma(-2, dot, |c|^2); T = (4D + 32) 2^-24 r^2 (1.001) + 2^-126, of
    which 2 (D + 4) 2^-24 r^2 is the reference's own distance error.
  * TF32 tensor-core screen (ckm_mma_screen.cuh): x = hi + mid with
    hi = tf32(x) (round to nearest, ties away), mid = x - hi read as TF32 by
    the tensor core (low 13 bits dropped); three chains (c_mid x_hi,
    c_hi x_mid, c_hi x_hi) added at the end; T = ((D + 8) 2^-22 +
    (2D + 8) 2^-24) r^2 (1.001), the score part being (D + 8) 2^-23 r^2.
  * Config 3's tensor-core label kernel (ckm_tc.cu): points and centroids
    scaled by powers of two and rounded once to fp16, one f32 chain, a T
    built from the measured rounding-error norms of both operands.
"""
import numpy as np
import pytest

U = 2.0 ** -24


def f32(v):
    return np.asarray(v, np.float64).astype(np.float32)


def fma32(a, b, c):
    """fma in FP32 (the product is exact in FP64; one rounding at the end)."""
    return f32(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def r_bound(X, C):
    """r as the kernels form it: (sqrt(|x|^2)(1 + 2^-16) + cm)(1 + 2^-20), with
    cm = sqrt(max |c|^2)(1 + 2^-16) and |c|^2 rounded once from FP64."""
    nx = np.zeros(X.shape[0], np.float32)
    for f in range(X.shape[1]):
        nx = fma32(X[:, f], X[:, f], nx)
    cn = f32((C.astype(np.float64) ** 2).sum(1))
    cm = np.float64(np.sqrt(np.float32(cn.max()))) * (1 + 2.0 ** -16)
    return (np.sqrt(nx.astype(np.float64)) * (1 + 2.0 ** -16) + cm) * (1 + 2.0 ** -20), cn


def exact_scores(X, C):
    Xd, Cd = X.astype(np.float64), C.astype(np.float64)
    return (Cd ** 2).sum(1)[None, :] - 2.0 * Xd @ Cd.T


def fp32_screen_scores(X, C, cn):
    n, D = X.shape
    ax = np.zeros((n, C.shape[0]), np.float32)
    ay = np.zeros((n, C.shape[0]), np.float32)
    for f in range(0, D, 2):
        ax = fma32(X[:, None, f], C[None, :, f], ax)
        ay = fma32(X[:, None, f + 1], C[None, :, f + 1], ay)
    dot = f32(ax.astype(np.float64) + ay)
    return fma32(-2.0, dot, cn[None, :])


def tf32_round(v):
    b = np.asarray(v, np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x1000) & 0xFFFFE000).astype(np.uint32).view(np.float32)


def tf32_trunc(v):
    return (np.asarray(v, np.float32).view(np.uint32) & np.uint32(0xFFFFE000)).view(np.float32)


def chain(a, b, steps):
    """Sum over features of a[:, None, f] * b[None, :, f] in FP32, 8 features per
    step (an m16n8k8 MMA), every product and addition rounded to FP32."""
    acc = np.zeros((a.shape[0], b.shape[0]), np.float32)
    for f in range(steps * 8):
        acc = f32(acc.astype(np.float64) + f32(a[:, None, f].astype(np.float64) * b[None, :, f]))
    return acc


def tf32_screen_scores(X, C, cn):
    D = X.shape[1]
    xh = tf32_round(X)
    xm = tf32_trunc(f32(X.astype(np.float64) - xh))
    ch = tf32_round(C)
    cmid = tf32_trunc(f32(C.astype(np.float64) - ch))
    p = chain(xh, cmid, D // 8)
    q = chain(xm, ch, D // 8)
    acc = chain(xh, ch, D // 8)
    total = f32(acc.astype(np.float64) + f32(p.astype(np.float64) + q))
    return fma32(-2.0, total, cn[None, :])


def sample(rng, D, scale, n=200, k=24):
    X = (rng.normal(0, 1, (n, D)) * scale).astype(np.float32)
    C = (rng.normal(0, 1, (k, D)) * scale).astype(np.float32)
    X[:4] = C[:4]                                  # points on centroids
    X[4:8] = (C[4:8] + C[8:12]) / 2                 # midway points
    X[8:12] *= np.float32(2.0 ** -30)               # tiny values
    return X, C


@pytest.mark.parametrize("D", [8, 16, 32, 64])
@pytest.mark.parametrize("scale", [1e-3, 1.0, 40.0, 2000.0])
def test_fp32_screen_score_error_within_its_share_of_T(D, scale):
    rng = np.random.default_rng(D * 7 + int(scale))
    X, C = sample(rng, D, scale)
    r, cn = r_bound(X, C)
    s = fp32_screen_scores(X, C, cn).astype(np.float64)
    T = ((4 * D + 32) * U * r * r + 2.0 ** -126) * 1.001
    share = (T - 2.0 * (D + 4) * U * r * r) / 2.0
    err = np.abs(s - exact_scores(X, C)).max(1)
    assert np.all(err <= share), float((err / share).max())


@pytest.mark.parametrize("D", [32, 64])
@pytest.mark.parametrize("scale", [1e-3, 1.0, 40.0, 2000.0])
def test_tf32_screen_score_error_within_its_share_of_T(D, scale):
    rng = np.random.default_rng(D * 11 + int(scale))
    X, C = sample(rng, D, scale, n=120, k=16)
    r, cn = r_bound(X, C)
    s = tf32_screen_scores(X, C, cn).astype(np.float64)
    share = (D + 8) * 2.0 ** -23 * r * r * 1.001
    err = np.abs(s - exact_scores(X, C)).max(1)
    assert np.all(err <= share), float((err / share).max())


def _scale_exponent(maxabs):
    """2^e * maxabs <= 2^15 (fp16 safe), e in [-60, 60] (ckm_tc.cu)."""
    if not maxabs > 0 or not np.isfinite(maxabs):
        return 0
    _, e = np.frexp(np.float32(maxabs))
    return int(min(60, max(-60, 15 - int(e))))


def tc_scores_and_threshold(X, C, d_pad):
    """The config-3 tensor-core label kernel's scores and its T per point
    (tc_points_convert_kernel, tc_centroid_stats/pack_kernel, tc_params_kernel),
    with the f32 accumulation of the MMA done sequentially in K = 16 blocks."""
    n, d = X.shape
    sx = 2.0 ** _scale_exponent(float(np.abs(X).max()))
    sc = 2.0 ** _scale_exponent(float(np.abs(C).max()))
    xs = f32(X.astype(np.float64) * sx)
    cs = f32(C.astype(np.float64) * sc)
    xh = xs.astype(np.float16).astype(np.float32)
    ch = cs.astype(np.float16).astype(np.float32)
    xn = np.sqrt((X.astype(np.float64) ** 2).sum(1) * (1 + 2.0 ** -14)) * (1 + 2.0 ** -20)
    xe = (np.sqrt(((xh.astype(np.float64) - xs) ** 2).sum(1) * (1 + 2.0 ** -14)) * (1 + 2.0 ** -20)
          + d * 2.0 ** -149) / sx
    csum = (C.astype(np.float64) ** 2).sum(1)
    cn = f32(csum)
    cm = np.sqrt(csum).max() * (1 + 2.0 ** -40)
    fm = ((np.sqrt(((ch.astype(np.float64) - cs) ** 2).sum(1)) * (1 + 2.0 ** -40) + d * 2.0 ** -149) / sc).max()
    acc = np.zeros((n, C.shape[0]), np.float32)
    for f in range(d):  # zero padding up to d_pad adds nothing
        acc = f32(acc.astype(np.float64) + f32(xh[:, None, f].astype(np.float64) * ch[None, :, f]))
    alpha = -2.0 / (sx * sc)
    s = fma32(alpha, acc, cn[None, :])
    gam, safety = 2.0 * d_pad * 2.0 ** -23, 1.0 + 2.0 ** -10
    t1 = (4.0 * fm + 4.0 * gam * (cm + fm)) * safety
    te = (4.0 * (cm + fm) + 4.0 * gam * (cm + fm)) * safety
    rho2 = 2.0 * (d + 2.0) * 2.0 ** -24 * 1.01 * safety
    t2 = 2.0 * 2.0 ** -23 * 1.01 * safety + rho2
    t0 = (d + 8.0) * 2.0 ** -146
    r = xn + cm
    T = (t2 * r * r + te * xe + t1 * xn + t0) * (1 + 2.0 ** -10)
    share = (T - rho2 * r * r) / 2.0
    return s.astype(np.float64), share


@pytest.mark.parametrize("d", [64, 128])
@pytest.mark.parametrize("scale", [1e-3, 2.0, 500.0])
def test_tensor_core_certificate_bounds_its_score_error(d, scale):
    """Config 3's fp16 certificate (single chain, measured rounding errors of
    the operands): the score error stays within half of T minus the
    reference's own distance error."""
    rng = np.random.default_rng(d + int(scale * 10))
    X = (rng.normal(0, 1, (120, d)) * scale).astype(np.float32)
    C = (rng.normal(0, 1, (32, d)) * scale).astype(np.float32)
    X[:4] = C[:4]
    X[4:8] *= np.float32(2.0 ** -12)  # small points next to large centroids
    s, share = tc_scores_and_threshold(X, C, d_pad=(d + 63) // 64 * 64)
    err = np.abs(s - exact_scores(X, C)).max(1)
    assert np.all(err <= share), float((err / share).max())


def _reference_labels(X, C):
    """The reference's FP32 distances and strict '<' argmin from cluster 0."""
    n, D = X.shape
    acc = np.zeros((n, C.shape[0]), np.float32)
    for f in range(D):
        t = f32(X[:, None, f].astype(np.float64) - C[None, :, f])
        acc = fma32(t, t, acc)
    best = np.full(n, np.finfo(np.float32).max, np.float32)
    lab = np.zeros(n, np.int64)
    for c in range(C.shape[0]):
        lt = acc[:, c] < best
        best = np.where(lt, acc[:, c], best)
        lab = np.where(lt, c, lab)
    return lab


def _near_ties(rng, D, n=600, k=16, spread=1e-3):
    centres = rng.uniform(-10, 10, (k - k // 4, D))
    C = np.concatenate([centres, centres[: k // 4] + rng.normal(0, spread, (k // 4, D))]).astype(np.float32)
    C[1] = C[0]
    X = (C[rng.integers(0, k, n)] + rng.normal(0, 1.0, (n, D))).astype(np.float32)
    return X, C


@pytest.mark.parametrize("D,screen", [(8, "fp32"), (32, "fp32"), (64, "fp32"), (32, "tf32"), (64, "tf32")])
def test_certified_labels_are_the_reference_labels(D, screen):
    """Near ties (duplicated and almost duplicated centroids): a label the
    screen certifies (m2 - m1 > T) is the reference's; the others go to the
    exact pass in the kernels."""
    rng = np.random.default_rng(D * 3 + len(screen))
    X, C = _near_ties(rng, D)
    ref = _reference_labels(X, C)
    r, cn = r_bound(X, C)
    if screen == "fp32":
        s = fp32_screen_scores(X, C, cn)
        T = ((4 * D + 32) * U * r * r + 2.0 ** -126) * 1.001
    else:
        s = tf32_screen_scores(X, C, cn)
        T = ((D + 8) * 2.0 ** -22 + (2 * D + 8) * 2.0 ** -24) * 1.001 * r * r + 2.0 ** -117 * (r + 1)
    order = np.argsort(s, axis=1, kind="stable")
    m1 = s[np.arange(len(X)), order[:, 0]].astype(np.float64)
    m2 = s[np.arange(len(X)), order[:, 1]].astype(np.float64)
    proved = (m2 - m1) > T
    assert np.all(order[proved, 0] == ref[proved])
    assert not np.any(proved[ref == 0])  # the duplicated pair 0 / 1 is never proved
    assert proved.mean() > 0.3
