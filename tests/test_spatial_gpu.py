"""Spatially ordered point sets: ckm_spatial_sort_f32 (a permutation of the
points in Z-order of their cells), ckm_fused_sorted_f32 (the fused
iteration with per-warp box pruning) and ckm_unpermute_u32.

Box pruning only skips clusters proved farther than another from every
point of a warp, so on any point order the labels must be the oracle's FP32
KmeansNaive labels bit for bit, masses exact, centroids within the fused
tolerance of the FP64 means."""
import numpy as np
import pytest

from conftest import blobs
from test_fused_gpu import check_centroids, to_dev

pytestmark = pytest.mark.gpu


def _sorted_set(ckm, cuda, P, n, d):
    import torch
    dP = to_dev(P, cuda)
    S, perm = ckm.spatial_sort(dP, n, d)
    torch.cuda.synchronize()
    return dP, S, perm


def test_spatial_sort_is_a_permutation(ckm, cuda):
    for n, d in [(1, 4), (7, 2), (1000, 1), (50001, 4), (70000, 3), (30000, 8), (20000, 16)]:
        P = blobs(n, d, 6, seed=n + d)
        dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
        pm = perm.cpu().numpy().view(np.uint32).astype(np.int64)
        assert np.array_equal(np.sort(pm), np.arange(n)), (n, d)
        X = P.reshape(d, n)
        assert np.array_equal(S.cpu().numpy().reshape(d, n), X[:, pm]), (n, d)


def test_spatial_sort_without_permutation(ckm, cuda):
    """perm = NULL: the same sorted points, no indices moved."""
    import torch
    for n, d in [(50001, 4), (33333, 3), (30000, 8), (4096 * 3, 2)]:
        P = blobs(n, d, 6, seed=n * d)
        dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
        S2, none = ckm.spatial_sort(dP, n, d, with_perm=False)
        torch.cuda.synchronize()
        assert none is None and torch.equal(S, S2), (n, d)


def test_spatial_sort_makes_warp_boxes_small(ckm, cuda):
    """After the sort, consecutive 256-point groups span a small part of the
    data's range (the property the pruning relies on)."""
    n, d = 1 << 18, 4
    P = blobs(n, d, 16, seed=3)
    dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
    X = S.cpu().numpy().reshape(d, n)
    span = X.max(1) - X.min(1)
    groups = X[:, : n // 256 * 256].reshape(d, -1, 256)
    g_span = groups.max(2) - groups.min(2)
    assert float(np.median(g_span / span[:, None])) < 0.2


@pytest.mark.parametrize("n,d,k,iters", [(1 << 17, 4, 16, 6), (60001, 2, 10, 5), (40000, 8, 32, 4),
                                         (30000, 3, 5, 4), (20000, 1, 7, 3), (25000, 4, 40, 3),
                                         (9000, 12, 6, 3), (100, 4, 16, 2)])
def test_fused_sorted_lockstep(ckm, oracle, cuda, n, d, k, iters):
    """k <= 32 and d <= 8 prune; k = 40 and d = 12 take the unpruned kernels."""
    import torch
    P = blobs(n, d, max(2, k // 2), seed=11 * n + d)
    dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
    Ps = S.cpu().numpy()
    pm = perm.cpu().numpy().view(np.uint32)
    C0 = oracle.first_x_f32(P, n, d, k)
    dC = [to_dev(C0, cuda), torch.zeros(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    out = torch.zeros(n, dtype=torch.int32, device=cuda)
    scr = ckm.new_scratch(d, k, cuda)
    for it in range(iters):
        Cin = dC[it % 2].cpu().numpy()
        ckm.fused_sorted(S, dC[it % 2], dC[(it + 1) % 2], dL, dM, scr, n, d, k, ckm.MODE_FINALIZE)
        ckm.unpermute(perm, dL, out, n)
        torch.cuda.synchronize()
        ref_sorted = oracle.label_f32(Ps, n, d, k, Cin)
        got = dL.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, ref_sorted), "iteration %d: %d labels differ" % (it, int((got != ref_sorted).sum()))
        ref = oracle.label_f32(P, n, d, k, Cin)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), ref)
        assert np.array_equal(ref[pm], ref_sorted)
        assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
        check_centroids(oracle, P, n, d, k, ref, dC[(it + 1) % 2].cpu().numpy())


def test_fused_sorted_ties_nan_inf_and_duplicates(ckm, oracle, cuda):
    """Exact ties between duplicated centroids (lowest index wins), a NaN
    centroid (never chosen), points with NaN or infinite coordinates, and many
    duplicate points: the pruned kernel keeps the oracle's labels."""
    import torch
    n, d, k = 40000, 4, 12
    P = blobs(n, d, 6, seed=21).reshape(d, n).copy()
    P[:, 100:600] = P[:, 100:101]          # duplicate points
    P[2, 1000] = np.nan
    P[0, 2000] = np.inf
    P[1, 3000] = -np.inf
    P = np.ascontiguousarray(P).reshape(-1)
    dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
    Ps = S.cpu().numpy()
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    C = np.nan_to_num(C, nan=0.0, posinf=1.0, neginf=-1.0)
    C[:, 5] = C[:, 2]          # exact tie: 2 wins
    C[:, 7] = np.nan           # never chosen
    C = np.ascontiguousarray(C).reshape(-1).astype(np.float32)
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    scr = ckm.new_scratch(d, k, cuda)
    ckm.fused_sorted(S, to_dev(C, cuda), dN, dL, dM, scr, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    ref = oracle.label_f32(Ps, n, d, k, C)
    got = dL.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, ref), "%d labels differ" % int((got != ref).sum())
    assert not np.any(got == 5) and not np.any(got == 7)


def test_spatial_rejects_bad_arguments(ckm, cuda):
    import torch
    t = torch.zeros(64, dtype=torch.float32, device=cuda)
    with pytest.raises(ckm.CkmError):
        ckm.spatial_sort(t, 4, 17)       # d > 16
    L = ckm.lib()
    assert L.ckm_spatial_sort_f32(4, 16, t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 16, None) != 0


def test_fused_sorted_without_labels(ckm, oracle, cuda):
    """labels = NULL: no labels written, the same masses and centroids (the
    strategies' intermediate iterations on a sorted copy)."""
    import torch
    n, d, k = 1 << 17, 4, 16
    P = blobs(n, d, 16, seed=21)
    dP, S, perm = _sorted_set(ckm, cuda, P, n, d)
    C0 = oracle.first_x_f32(P, n, d, k)
    out = []
    for with_labels in (True, False):
        dC = to_dev(C0, cuda)
        dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
        dL = torch.full((n,), -1, dtype=torch.int32, device=cuda)
        dM = torch.zeros(k, dtype=torch.int32, device=cuda)
        sc = ckm.new_scratch(d, k, cuda)
        ckm.fused_sorted(S, dC, dN, dL if with_labels else None, dM, sc, n, d, k, ckm.MODE_FINALIZE)
        torch.cuda.synchronize()
        out.append((dN.cpu().numpy(), dM.cpu().numpy(), dL.cpu().numpy()))
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.all(out[1][2] == -1)                      # untouched
    ref = oracle.label_f32(P, n, d, k, C0)
    assert np.array_equal(out[0][2].view(np.uint32), ref[perm.cpu().numpy().view(np.uint32)])
