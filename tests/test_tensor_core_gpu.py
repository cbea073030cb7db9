"""Tensor-core fused iteration (ckm_tc_fused_f32): fp16 (or bf16) distances on
tcgen05 with certified labels and exact FP32 recheck of near-ties.  The
labels must be bit-exact against the oracle's restatement of the reference
arithmetic (kmeans_naive.cpp:48-63) -- the certificate plus recheck is what
makes a 16-bit GEMM give reference labels -- masses exact, centroids within
the fused tolerance of the FP64 means."""
import numpy as np
import pytest

from conftest import blobs
from test_fused_gpu import check_centroids, to_dev

pytestmark = pytest.mark.gpu


def run_tc(ckm, cuda, P, n, d, k, C, iters=1, precision="fp16"):
    import torch
    dP = to_dev(P, cuda)
    tcp = ckm.TensorCorePoints(dP, n, d, precision=precision)
    bufs = [to_dev(C, cuda), torch.zeros(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    stats = torch.zeros(2, dtype=torch.int32, device=cuda)
    hist = []
    for it in range(iters):
        Cin = bufs[it % 2].cpu().numpy()
        ckm.tc_fused(dP, tcp, bufs[it % 2], bufs[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE, stats)
        torch.cuda.synchronize()
        hist.append((Cin, dL.cpu().numpy().view(np.uint32).copy(), dM.cpu().numpy().view(np.uint32).copy(),
                     bufs[(it + 1) % 2].cpu().numpy().copy(), stats.cpu().numpy().copy()))
    return hist


def check_iter(oracle, P, n, d, k, Cin, lab, mass, Cout):
    ref = oracle.label_f32(P, n, d, k, Cin)
    assert np.array_equal(lab, ref), "%d labels differ" % int((lab != ref).sum())
    assert np.array_equal(mass, oracle.mass_u32(ref, k))
    check_centroids(oracle, P, n, d, k, ref, Cout)


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
@pytest.mark.parametrize("n,d,k,iters", [(20000, 128, 1024, 2), (9999, 64, 300, 3), (5000, 100, 50, 3),
                                         (3000, 256, 256, 2), (4097, 32, 40, 3)])
def test_tc_lockstep_matches_oracle(ckm, oracle, cuda, n, d, k, iters, precision):
    """fp16 and bf16 operands: either way the certificate (built from the
    operands' measured rounding errors) and the exact resolution give the
    reference's labels."""
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, max(2, k // 4), seed=n + d + k, spread=4.0, sigma=0.5)
    C0 = oracle.first_x_f32(P, n, d, k)
    for Cin, lab, mass, Cout, st in run_tc(ckm, cuda, P, n, d, k, C0, iters, precision):
        assert st[1] == 0, "device wait ran out"
        check_iter(oracle, P, n, d, k, Cin, lab, mass, Cout)


def test_tc_ties_and_empty_clusters(ckm, oracle, cuda):
    n, d, k = 6000, 64, 64
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, 16, seed=77, spread=3.0)
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    C[:, 9] = C[:, 5]          # exact duplicate: the lower index wins among the in-kernel candidates
    C[:, 20] = np.nan          # empty cluster from a previous iteration: never chosen
    dup = list(range(40, 52))  # twelve more copies of cluster 7: more ties than the kernel keeps,
    C[:, dup] = C[:, [7]]      # so those points go to the full exact recheck
    C = np.ascontiguousarray(C).reshape(-1)
    (Cin, lab, mass, Cout, st), = run_tc(ckm, cuda, P, n, d, k, C, 1)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(lab, ref)
    assert not np.any(lab == 9) and not np.any(lab == 20) and not np.any(np.isin(lab, dup))
    assert np.any(lab == 5) and np.any(lab == 7)
    assert st[0] > 0, "more tied clusters than candidates must send their points to the exact recheck"


@pytest.mark.parametrize("scale,offset", [(1e6, 0.0), (1e-6, 0.0), (1.0, -3e3), (3e-30, 1e-29)])
def test_tc_extreme_magnitudes(ckm, oracle, cuda, scale, offset):
    """Power-of-two operand scaling keeps fp16 in range for any magnitude;
    labels stay the reference's."""
    n, d, k = 8192, 48, 96
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = (blobs(n, d, 24, seed=5, spread=4.0, sigma=0.6).astype(np.float64) * scale + offset).astype(np.float32)
    C0 = oracle.first_x_f32(P, n, d, k)
    for Cin, lab, mass, Cout, st in run_tc(ckm, cuda, P, n, d, k, C0, 2):
        assert st[1] == 0
        check_iter(oracle, P, n, d, k, Cin, lab, mass, Cout)


@pytest.mark.parametrize("d", [1, 3, 7, 200])
def test_tc_small_and_odd_feature_counts(ckm, oracle, cuda, d):
    n, k = 6001, 150
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, 40, seed=d, spread=5.0, sigma=0.7)
    C0 = oracle.first_x_f32(P, n, d, k)
    for Cin, lab, mass, Cout, st in run_tc(ckm, cuda, P, n, d, k, C0, 2):
        assert st[1] == 0
        check_iter(oracle, P, n, d, k, Cin, lab, mass, Cout)


def test_tc_nan_points_get_label_zero(ckm, oracle, cuda):
    """A point with a NaN coordinate has NaN distances: the reference keeps
    label 0 (nothing is below FLT_MAX)."""
    n, d, k = 3000, 32, 64
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, 16, seed=11).reshape(d, n)
    P[3, [17, 1000, 2999]] = np.nan
    P = np.ascontiguousarray(P).reshape(-1)
    C = oracle.first_x_f32(P, n, d, k)
    (Cin, lab, mass, Cout, st), = run_tc(ckm, cuda, P, n, d, k, C, 1)
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(lab, ref)
    assert lab[17] == 0 and lab[1000] == 0 and lab[2999] == 0
    assert np.array_equal(mass, oracle.mass_u32(ref, k))


def test_tc_defer_then_finalize_over_chunks(ckm, oracle, cuda):
    """CKM_MODE_DEFER over two point chunks, then ckm_finalize_f32: the same
    centroids and masses as one call over all points (the buffered pipeline's
    use of the fused functor)."""
    import torch
    n, d, k = 12000, 64, 200
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, 50, seed=21, spread=4.0, sigma=0.5)
    C = oracle.first_x_f32(P, n, d, k)
    ref = oracle.label_f32(P, n, d, k, C)
    Pm = P.reshape(d, n)
    h = 7001
    dC = to_dev(C, cuda)
    S = ckm.new_scratch(d, k, cuda)
    labs = []
    for lo, hi in ((0, h), (h, n)):
        part = np.ascontiguousarray(Pm[:, lo:hi]).reshape(-1)
        m = hi - lo
        dP = to_dev(part, cuda)
        tcp = ckm.TensorCorePoints(dP, m, d)
        dL = torch.zeros(m, dtype=torch.int32, device=cuda)
        ckm.tc_fused(dP, tcp, dC, dC, dL, None, S, m, d, k, ckm.MODE_DEFER)
        torch.cuda.synchronize()
        labs.append(dL.cpu().numpy().view(np.uint32).copy())
    lab = np.concatenate(labs)
    assert np.array_equal(lab, ref)
    out = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    ckm.finalize(out, dM, S, d, k)
    torch.cuda.synchronize()
    assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
    check_centroids(oracle, P, n, d, k, ref, out.cpu().numpy())


def test_tc_sorted_point_set_keeps_caller_order(ckm, oracle, cuda):
    """ckm_tc_sort_points reorders the prepared set by the last labels; the
    following iterations still return labels in the caller's point order,
    equal to the oracle's, and the same centroids as the unsorted set."""
    import torch
    n, d, k = 30011, 96, 300
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, 60, seed=31, spread=4.0, sigma=0.6)
    C0 = oracle.first_x_f32(P, n, d, k)
    dP = to_dev(P, cuda)
    tcp = ckm.TensorCorePoints(dP, n, d)
    bufs = [to_dev(C0, cuda), torch.zeros(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    for it in range(4):
        Cin = bufs[it % 2].cpu().numpy()
        ckm.tc_fused(dP, tcp, bufs[it % 2], bufs[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
        torch.cuda.synchronize()
        check_iter(oracle, P, n, d, k, Cin, dL.cpu().numpy().view(np.uint32), dM.cpu().numpy().view(np.uint32),
                   bufs[(it + 1) % 2].cpu().numpy())
        if it < 2:
            tcp.sort(k)   # sorted by the labels of this iteration (twice: a sorted set sorts again)
