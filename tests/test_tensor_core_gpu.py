"""Tensor-core fused iteration (ckm_tc_fused_f32): bf16 distances on
tcgen05 with certified labels and exact FP32 recheck of near-ties.  The
labels must be bit-exact against the oracle's restatement of the reference
arithmetic (kmeans_naive.cpp:48-63) -- the certificate plus recheck is what
makes a bf16 GEMM give reference labels -- masses exact, centroids within
the fused tolerance of the FP64 means."""
import numpy as np
import pytest

from conftest import blobs
from test_fused_gpu import check_centroids, to_dev

pytestmark = pytest.mark.gpu


def run_tc(ckm, cuda, P, n, d, k, C, iters=1):
    import torch
    dP = to_dev(P, cuda)
    tcp = ckm.TensorCorePoints(dP, n, d)
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


@pytest.mark.parametrize("n,d,k,iters", [(20000, 128, 1024, 2), (9999, 64, 300, 3), (5000, 100, 50, 3),
                                         (3000, 256, 256, 2), (4097, 32, 40, 3)])
def test_tc_lockstep_matches_oracle(ckm, oracle, cuda, n, d, k, iters):
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = blobs(n, d, max(2, k // 4), seed=n + d + k, spread=4.0, sigma=0.5)
    C0 = oracle.first_x_f32(P, n, d, k)
    for Cin, lab, mass, Cout, st in run_tc(ckm, cuda, P, n, d, k, C0, iters):
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
