"""Parity of the fused single-pass kernel (ckm_fused_*) with the oracle.

Gate 1 (per iteration): with identical input centroids the labels are
bit-exact against the oracle's FP32 restatement of KmeansNaive
(kmeans_naive.cpp:48-63), the masses are exact, and the new centroids are
within CENTROID_RTOL of the FP64 means of the same labels.
Gate 2 (lockstep): over many iterations, every iteration's GPU labels equal
the oracle's labels for that iteration's GPU input centroids.
"""
import numpy as np
import pytest

from conftest import blobs

# Centroid tolerance against FP64 means of the same labels: per-CTA FP32
# partial sums merged in FP64, one rounding to FP32 at the end.
CENTROID_RTOL = 2e-6
CENTROID_ATOL_SCALE = 2e-6  # times max |x| of the data set

pytestmark = pytest.mark.gpu


def to_dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def run_fused_once(ckm, cuda, P, n, d, k, C, mode=1):
    import torch
    dP = to_dev(P, cuda)
    dC = to_dev(C.astype(np.float32), cuda)
    dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.fused(dP, dC, dN, dL, dM, S, n, d, k, mode)
    torch.cuda.synchronize()
    return (dN.cpu().numpy(), dM.cpu().numpy().view(np.uint32), dL.cpu().numpy().view(np.uint32), S)


def check_centroids(oracle, P, n, d, k, labels, got):
    sums, masses = oracle.sums_f64(P, n, d, k, labels)
    with np.errstate(invalid="ignore", divide="ignore"):
        ref = sums / np.tile(masses.astype(np.float64), d)
    scale = float(np.abs(P).max()) if P.size else 1.0
    empty = np.tile(masses == 0, d)
    assert np.all(np.isnan(got[empty])), "empty clusters must give NaN centroids"
    g, r = got[~empty].astype(np.float64), ref[~empty]
    err = np.abs(g - r)
    tol = CENTROID_RTOL * np.abs(r) + CENTROID_ATOL_SCALE * scale
    assert np.all(err <= tol), "max centroid error %g (tol %g)" % (err.max(), tol[np.argmax(err - tol)])


SHAPES = [
    # (n, d, k) -- low-d kernel private table, shared table, ragged n, generic path
    (4096, 4, 16),
    (4099, 4, 10),
    (10007, 1, 5),
    (20000, 2, 7),
    (12345, 3, 9),
    (33333, 5, 12),
    (8191, 6, 4),
    (9000, 7, 3),
    (65536, 8, 10),
    (7777, 12, 6),
    (50000, 16, 64),
    (30000, 4, 200),
    (5000, 2, 1000),
    (3000, 20, 17),
    (2047, 33, 40),
    (1000, 128, 64),
    (100, 4, 1),
    # fixed-d rows kernel (d = 32, 64): cluster counts not a multiple of four,
    # 256-thread and 512-thread CTAs (by table size), one cluster
    (20011, 32, 7),
    (9000, 64, 5),
    (6000, 64, 300),
    (7000, 32, 600),
    (3000, 64, 1),
    (4100, 32, 2),
    # rows kernel on the tensor-core screen (d = 32 with k >= 64, d = 64 with
    # k >= 32, while the TF32 fragments fit in shared memory)
    (9000, 64, 40),
    (8000, 32, 100),
    (5000, 64, 200),
    (3001, 32, 64),
]


@pytest.mark.parametrize("n,d,k", SHAPES)
def test_fused_one_iteration_matches_oracle(ckm, oracle, cuda, n, d, k):
    P = blobs(n, d, max(2, k // 2), seed=n + 31 * d + k)
    C = oracle.first_x_f32(P, n, d, k)
    newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
    ref_labels = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(labels, ref_labels), "labels differ at %d points" % int((labels != ref_labels).sum())
    assert np.array_equal(masses, oracle.mass_u32(ref_labels, k))
    check_centroids(oracle, P, n, d, k, ref_labels, newC)


@pytest.mark.parametrize("n,d,k,iters", [(1 << 16, 4, 16, 20), (40000, 2, 10, 15), (30001, 8, 24, 10),
                                         (20000, 20, 12, 8), (16384, 64, 40, 6), (12000, 32, 13, 6),
                                         (12000, 32, 90, 5)])
def test_fused_lockstep_iterations(ckm, oracle, cuda, n, d, k, iters):
    import torch
    P = blobs(n, d, k, seed=7 * n + d)
    C0 = oracle.first_x_f32(P, n, d, k)
    dP = to_dev(P, cuda)
    dC = [to_dev(C0, cuda), torch.zeros(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    for it in range(iters):
        Cin = dC[it % 2].cpu().numpy()
        ckm.fused(dP, dC[it % 2], dC[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
        torch.cuda.synchronize()
        labels = dL.cpu().numpy().view(np.uint32)
        ref = oracle.label_f32(P, n, d, k, Cin)
        assert np.array_equal(labels, ref), "iteration %d: %d labels differ" % (it, int((labels != ref).sum()))
        assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
        check_centroids(oracle, P, n, d, k, ref, dC[(it + 1) % 2].cpu().numpy())


def test_ties_pick_lowest_index_and_nan_never_wins(ckm, oracle, cuda):
    # duplicate centroids tie exactly: the lowest index must win; an empty
    # cluster (NaN centroid) must never be chosen afterwards
    n, d, k = 2048, 4, 6
    P = blobs(n, d, 3, seed=5)
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    C[:, 3] = C[:, 1]           # exact tie between clusters 1 and 3
    C[:, 5] = 1e6               # far away: stays empty -> NaN next iteration
    C = C.reshape(-1)
    newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(labels, ref)
    assert masses[3] == 0 and masses[5] == 0
    assert np.all(np.isnan(newC.reshape(d, k)[:, [3, 5]]))
    newC2, masses2, labels2, _ = run_fused_once(ckm, cuda, P, n, d, k, newC)
    ref2 = oracle.label_f32(P, n, d, k, newC)
    assert np.array_equal(labels2, ref2)
    assert not np.any(np.isin(labels2, [3, 5]))


@pytest.mark.parametrize("d,k", [(32, 9), (64, 6), (64, 260), (64, 40), (32, 70)])
def test_rows_kernel_ties_nan_and_labeling(ckm, oracle, cuda, d, k):
    """d = 32 / 64 (fixed-d rows kernel): exact ties inside and across the
    four-cluster steps pick the lowest index, a NaN centroid never wins, and
    the labeling pass gives the fused pass's labels."""
    import torch
    n = 5000
    P = blobs(n, d, 4, seed=d + k)
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    C[:, 2] = C[:, 1]            # tie inside one step of four
    C[:, 4] = C[:, 3]            # tie across two steps
    C[:, k - 1] = C[:, 0]        # tie with the remainder loop (k % 4 != 0)
    C[:, 5] = np.nan
    C = C.reshape(-1)
    newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(labels, ref), "labels differ at %d points" % int((labels != ref).sum())
    assert not np.any(np.isin(labels, [2, 4, 5, k - 1]))
    assert np.array_equal(masses, oracle.mass_u32(ref, k))
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    ckm.labeling(to_dev(P, cuda), to_dev(C, cuda), dL, n, d, k)
    torch.cuda.synchronize()
    assert np.array_equal(dL.cpu().numpy().view(np.uint32), ref)


@pytest.mark.parametrize("d,case,k", [(32, "offset", 24), (64, "offset", 24), (64, "huge", 24), (32, "inf", 24),
                                      (64, "offset", 48), (32, "offset", 80), (64, "huge", 40), (32, "inf", 72)])
def test_screen_fallback_keeps_reference_labels(ckm, oracle, cuda, d, case, k):
    """d = 32 / 64 label through the certified screen.  Points it cannot prove
    are labelled with the exact loop: data far from the origin (the rounding
    bound grows with |x| + max|c|, so many points fall back), a centroid so
    large that (|x| + max|c|)^2 >= 2^120 (every point falls back), and an
    infinite centroid (every point falls back; that cluster never wins).
    k = 24: FP32 screen; k = 40..80: tensor-core screen."""
    n = 6000
    P = blobs(n, d, 8, seed=d + len(case))
    if case == "offset":
        P = (P + np.float32(3000.0)).astype(np.float32)
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    if case == "huge":
        C[:, 4] = 1e30
    elif case == "inf":
        C[0, 4] = np.inf
    C = C.reshape(-1)
    newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(labels, ref), "labels differ at %d points" % int((labels != ref).sum())
    assert np.array_equal(masses, oracle.mass_u32(ref, k))


def test_accumulate_mode_adds_into_outputs(ckm, oracle, cuda):
    """Reference FusedFunction contract: += into new_centroids and masses."""
    import torch
    n, d, k = 10000, 4, 8
    P = blobs(n, d, k, seed=11)
    C = oracle.first_x_f32(P, n, d, k)
    dP, dC = to_dev(P, cuda), to_dev(C, cuda)
    dN = torch.full((k * d,), 1.5, dtype=torch.float32, device=cuda)
    dM = torch.full((k,), 3, dtype=torch.int32, device=cuda)
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.fused(dP, dC, dN, dL, dM, S, n, d, k, ckm.MODE_ACCUMULATE)
    torch.cuda.synchronize()
    ref_l = oracle.label_f32(P, n, d, k, C)
    sums, masses = oracle.sums_f64(P, n, d, k, ref_l)
    assert np.array_equal(dM.cpu().numpy(), masses.astype(np.int64) + 3)
    got = dN.cpu().numpy().astype(np.float64) - 1.5
    assert np.allclose(got, sums, rtol=1e-5, atol=1e-2)
    # scratch must be left zeroed: a second FINALIZE call gives plain means
    dN2 = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    ckm.fused(dP, dC, dN2, dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    check_centroids(oracle, P, n, d, k, ref_l, dN2.cpu().numpy())


def test_defer_then_finalize_over_chunks(ckm, oracle, cuda):
    """Chunked accumulation (buffered strategies): DEFER per chunk, one finalize."""
    import torch
    n, d, k = 50000, 4, 16
    P = blobs(n, d, k, seed=12)
    C = oracle.first_x_f32(P, n, d, k)
    X = P.reshape(d, n)
    dC = to_dev(C, cuda)
    S = ckm.new_scratch(d, k, cuda)
    labels = []
    for lo, hi in [(0, 12345), (12345, 40000), (40000, n)]:
        chunk = np.ascontiguousarray(X[:, lo:hi]).reshape(-1)
        dP = to_dev(chunk, cuda)
        dL = torch.zeros(hi - lo, dtype=torch.int32, device=cuda)
        ckm.fused(dP, dC, None, dL, None, S, hi - lo, d, k, ckm.MODE_DEFER)
        torch.cuda.synchronize()
        labels.append(dL.cpu().numpy().view(np.uint32))
    dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    ckm.finalize(dN, dM, S, d, k)
    torch.cuda.synchronize()
    lab = np.concatenate(labels)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(lab, ref)
    assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
    check_centroids(oracle, P, n, d, k, ref, dN.cpu().numpy())


def test_unaligned_views_use_scalar_path(ckm, oracle, cuda):
    """Points/labels that are not 16-byte aligned must still be exact."""
    import torch
    n, d, k = 5001, 4, 9
    P = blobs(n, d, k, seed=13)
    C = oracle.first_x_f32(P, n, d, k)
    base = torch.zeros(n * d + 1, dtype=torch.float32, device=cuda)
    base[1:] = to_dev(P, cuda)
    dP = base[1:]
    lbase = torch.zeros(n + 1, dtype=torch.int32, device=cuda)
    dL = lbase[1:]
    dC = to_dev(C, cuda)
    dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.fused(dP, dC, dN, dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(dL.cpu().numpy().view(np.uint32), ref)
    check_centroids(oracle, P, n, d, k, ref, dN.cpu().numpy())


def test_fused_f64_matches_oracle(ckm, oracle, cuda):
    import torch
    n, d, k = 6000, 3, 7
    P = blobs(n, d, k, seed=14).astype(np.float64)
    C = oracle.first_x_f32(P.astype(np.float32), n, d, k).astype(np.float64)
    dP, dC = to_dev(P, cuda), to_dev(C, cuda)
    dN = torch.zeros(k * d, dtype=torch.float64, device=cuda)
    dL = torch.zeros(n, dtype=torch.int64, device=cuda)
    dM = torch.zeros(k, dtype=torch.int64, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.fused(dP, dC, dN, dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    ref_l = oracle.label_f64(P, n, d, k, C)
    assert np.array_equal(dL.cpu().numpy().view(np.uint64), ref_l)
    refC, refM, _ = oracle.lloyd_f64(P, n, d, k, 1, C)
    assert np.array_equal(dM.cpu().numpy().view(np.uint64), refM)
    assert np.allclose(dN.cpu().numpy(), refC, rtol=1e-13, atol=1e-12)


def test_zero_points_finalize_gives_nan(ckm, cuda):
    import torch
    d, k = 4, 5
    dC = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dM = torch.ones(k, dtype=torch.int32, device=cuda)
    dP = torch.zeros(4, dtype=torch.float32, device=cuda)
    dL = torch.zeros(4, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.fused(dP, dC, dN, dL, dM, S, 0, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    assert torch.isnan(dN).all() and (dM == 0).all()


def test_invalid_arguments_are_rejected(ckm, cuda):
    import torch
    dP = torch.zeros(16, dtype=torch.float32, device=cuda)
    S = ckm.new_scratch(4, 4, cuda)
    with pytest.raises(ckm.CkmError) as e:
        ckm.fused(dP, dP, dP, dP, dP, S, 4, 0, 4)  # d = 0
    assert e.value.status == -1
    small = torch.zeros(8, dtype=torch.uint8, device=cuda)
    with pytest.raises(ckm.CkmError) as e:
        ckm.fused(dP, dP, dP, dP, dP, small, 4, 4, 4)
    assert e.value.status == -3


# d = 32 / 64, FINALIZE: ckm_fused_f32 runs one job on the batched kernel's
# tensor-core path (tcgen05, certified screen, exact resolution of unproved
# points) when n >= 2^20 and k >= 128; CKM_FUSED_UMMA=1 forces it at any n and
# 16 <= k <= 256, =0 keeps the rows kernel.
UMMA_ROUTE = [(1 << 20, 64, 128, None), (1 << 20, 32, 256, None), (100003, 32, 40, "1"), (70001, 64, 256, "1"),
              (65536, 32, 16, "1"), (131072, 32, 255, "1")]


@pytest.mark.parametrize("n,d,k,force", UMMA_ROUTE)
def test_fused_tensor_core_route_matches_oracle(ckm, oracle, cuda, monkeypatch, n, d, k, force):
    if force:
        monkeypatch.setenv("CKM_FUSED_UMMA", force)
    P = blobs(n, d, max(2, k // 2), seed=n + 31 * d + k)
    C = oracle.first_x_f32(P, n, d, k)
    newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(labels, ref), "labels differ at %d points" % int((labels != ref).sum())
    assert np.array_equal(masses, oracle.mass_u32(ref, k))
    check_centroids(oracle, P, n, d, k, ref, newC)


def test_fused_tensor_core_route_lockstep(ckm, oracle, cuda, monkeypatch):
    """Several iterations on one scratch buffer: the route's records in the
    scratch are rebuilt every call and its sums re-zeroed."""
    import torch
    monkeypatch.setenv("CKM_FUSED_UMMA", "1")
    n, d, k, iters = 100000, 64, 96, 5
    P = blobs(n, d, k, seed=17)
    C0 = oracle.first_x_f32(P, n, d, k)
    dP = to_dev(P, cuda)
    dC = [to_dev(C0, cuda), torch.zeros(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    for it in range(iters):
        Cin = dC[it % 2].cpu().numpy()
        ckm.fused(dP, dC[it % 2], dC[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
        torch.cuda.synchronize()
        ref = oracle.label_f32(P, n, d, k, Cin)
        assert np.array_equal(dL.cpu().numpy().view(np.uint32), ref), "iteration %d" % it
        assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
        check_centroids(oracle, P, n, d, k, ref, dC[(it + 1) % 2].cpu().numpy())
    # the scratch is back to zero for the next caller (sums and masses)
    assert not torch.any(S[:ckm.scratch_bytes(d, k) - 4096 - 256] != 0)


@pytest.mark.parametrize("force", ["1", "0"])
def test_fused_tensor_core_route_forced_ties_nan(ckm, oracle, cuda, monkeypatch, force):
    """The route forced on at small n (CKM_FUSED_UMMA=1) and off (=0): exact
    ties pick the lowest index and a NaN centroid never wins either way."""
    monkeypatch.setenv("CKM_FUSED_UMMA", force)
    for d, k in [(32, 40), (64, 17), (64, 256)]:
        n = 6000
        P = blobs(n, d, 6, seed=d + k)
        C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
        C[:, 2] = C[:, 1]
        C[:, 9] = C[:, 3]
        C[:, 5] = np.nan
        C = np.ascontiguousarray(C).reshape(-1)
        newC, masses, labels, _ = run_fused_once(ckm, cuda, P, n, d, k, C)
        ref = oracle.label_f32(P, n, d, k, C)
        assert np.array_equal(labels, ref), (d, k, int((labels != ref).sum()))
        assert not np.any(np.isin(labels, [2, 5, 9]))
        assert np.array_equal(masses, oracle.mass_u32(ref, k))
        check_centroids(oracle, P, n, d, k, ref, newC)
