"""Parity at the benchmark configurations' own sizes, against the oracle and
an FP64 oracle.

* Plain Lloyd, n = 2^20, d = 4, k = 10, 30 iterations (10 isotropic blobs,
  centres U[-10, 10]^4, sigma 1, equal weights, shuffled from seed 42;
  initial centroids the first k points, kmeans_initializer.cpp:29-39), end to
  end through ckm_kmeans_run_f32 for the single-stage and three-stage
  pipelines (kmeans_single_stage.hpp:52-172, kmeans_three_stage.hpp:66-243).
  Labels against the oracle's FP32 KmeansNaive run (and the reference's own
  build when present); every mismatch is adjudicated in FP64 against the
  derived near-tie bound (tests/parity.py).  Centroids against an FP64
  Lloyd run from the same start: relative error <= 1e-5.
* HBM-scale Lloyd (n = 2^28, d = 4, k = 16, 16 blobs, sigma U[0.5, 2]): the
  first 2^24 points of the same generated set in lockstep, on the caller's
  order (ckm_fused_f32) and on the spatial order (ckm_spatial_sort_f32 +
  ckm_fused_sorted_f32) -- every iteration's labels bit-exact against the
  oracle from the same input centroids, masses exact, centroids within the
  fused tolerance of the FP64 means; and the full 2^28 points through
  size-independent properties: both orders give the same masses and
  centroids, the masses sum to n, and a 2^20-point sample of the labels equals
  the oracle's.
* The same workload end to end at its size through ckm_kmeans_run_f32 with
  host buffers (50 iterations): masses against the label counts, centroids
  against the FP64 means of the labels, a 2^20-point sample of the last
  iteration's labels against the oracle.
* Tensor-core Lloyd at its size (n = 2^24, d = 128, k = 1024): two
  iterations, a 16384-point sample of the labels against the oracle, masses
  against the label counts, centroids against the FP64 means of the labels.
* Batched jobs at their size (4096 jobs, 196 M points): one step, every
  job's masses and centroids against its labels in FP64, every 64th job's
  labels against the oracle.
"""
import numpy as np
import pytest

import parity
from conftest import blobs
from test_fused_gpu import check_centroids

pytestmark = pytest.mark.gpu

FP64_REL_TOL = 1e-5


@pytest.mark.parametrize("pipeline", ["single_stage", "three_stage"])
def test_config1_end_to_end(ckm, oracle, cuda, pipeline):
    n, d, k, iters = 1 << 20, 4, 10, 30
    P = blobs(n, d, k, seed=42)
    C0 = oracle.first_x_f32(P, n, d, k)
    C, M, L, info = ckm.kmeans_run(P, d, k, iters, C0, pipeline=pipeline)
    assert info.iterations == iters
    L = L.view(np.uint32)
    Cr, Mr, Lr = oracle.lloyd_f32(P, n, d, k, iters, C0)
    if oracle.ref_available():
        # the oracle is the reference's arithmetic, bit for bit, at this size too
        Cx, Mx, Lx = oracle.ref_naive_f32(P, n, d, k, iters, C0)
        assert np.array_equal(Lx, Lr) and np.array_equal(Mx, Mr)
        assert np.array_equal(Cx.view(np.uint32), Cr.view(np.uint32))

    def ours_prev():
        return ckm.kmeans_run(P, d, k, iters - 1, C0, pipeline=pipeline)[0]

    prev = None
    if np.any(L != Lr):
        prev = ours_prev()
        parity.adjudicate(P, n, d, k, L, Lr, prev, oracle.lloyd_f32(P, n, d, k, iters - 1, C0)[0])
    assert np.array_equal(M, oracle.mass_u32(L, k))
    check_centroids(oracle, P, n, d, k, L, C)

    # against the FP64 oracle (FP64 distances and sums, the same FP32 points)
    C64, M64, L64 = oracle.lloyd_fp64_of_f32(P, n, d, k, iters, C0)
    if np.any(L != L64):
        prev = ours_prev() if prev is None else prev
        parity.adjudicate(P, n, d, k, L, L64, prev, oracle.lloyd_fp64_of_f32(P, n, d, k, iters - 1, C0)[0])
    assert parity.rel_centroid_error(C, C64) <= FP64_REL_TOL


def _c2a(ckm, cuda, n, first_point=0):
    import torch
    P = torch.empty(n * 4, dtype=torch.float32, device=cuda)
    ckm.generate_mixture(P, n, 4, 16, 42, sigma=(0.5, 2.0), first_point=first_point)
    return P


@pytest.mark.parametrize("order", ["caller", "spatial"])
def test_config2a_lockstep_2p24(ckm, oracle, cuda, order):
    import torch
    n, d, k, iters = 1 << 24, 4, 16, 4
    dP = _c2a(ckm, cuda, n)
    P = dP.cpu().numpy()
    C = [dP.view(d, n)[:, :k].reshape(-1).clone(), torch.empty(k * d, dtype=torch.float32, device=cuda)]
    dL = torch.empty(n, dtype=torch.int32, device=cuda)
    dM = torch.empty(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    if order == "spatial":
        dPs, perm = ckm.spatial_sort(dP, n, d)
        torch.cuda.synchronize()
        perm_h = perm.cpu().numpy().view(np.uint32)
        assert np.array_equal(np.sort(perm_h), np.arange(n, dtype=np.uint32))
        assert np.array_equal(dPs.cpu().numpy().reshape(d, n), P.reshape(d, n)[:, perm_h])
    for it in range(iters):
        Cin = C[it % 2].cpu().numpy()
        if order == "spatial":
            ckm.fused_sorted(dPs, C[it % 2], C[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
        else:
            ckm.fused(dP, C[it % 2], C[(it + 1) % 2], dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
        torch.cuda.synchronize()
        ref = oracle.label_f32(P, n, d, k, Cin)
        L = dL.cpu().numpy().view(np.uint32)
        assert np.array_equal(L, ref[perm_h] if order == "spatial" else ref), "iteration %d" % it
        assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
        check_centroids(oracle, P, n, d, k, ref, C[(it + 1) % 2].cpu().numpy())


def test_config2a_full_size_properties(ckm, oracle, cuda):
    """n = 2^28: one iteration on each order from the first-k centroids."""
    import torch
    n, d, k = 1 << 28, 4, 16
    dP = _c2a(ckm, cuda, n)
    C0 = dP.view(d, n)[:, :k].reshape(-1).clone()
    out = {}
    dL = torch.empty(n, dtype=torch.int32, device=cuda)
    dM = torch.empty(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    Cn = torch.empty(k * d, dtype=torch.float32, device=cuda)
    ckm.fused(dP, C0, Cn, dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    out["caller"] = (dM.cpu().numpy().view(np.uint32).copy(), Cn.cpu().numpy().copy())
    rng = np.random.default_rng(7)
    sample = np.sort(rng.choice(n, size=1 << 20, replace=False))
    Xs = np.ascontiguousarray(dP.view(d, n)[:, torch.from_numpy(sample).to(cuda)].cpu().numpy()).reshape(-1)
    ref_sample = oracle.label_f32(Xs, len(sample), d, k, C0.cpu().numpy())
    assert np.array_equal(dL.cpu().numpy().view(np.uint32)[sample], ref_sample)
    dPs, perm = ckm.spatial_sort(dP, n, d)
    del dP
    ckm.fused_sorted(dPs, C0, Cn, dL, dM, S, n, d, k, ckm.MODE_FINALIZE)
    torch.cuda.synchronize()
    out["spatial"] = (dM.cpu().numpy().view(np.uint32).copy(), Cn.cpu().numpy().copy())
    Ls = torch.empty_like(dL)
    ckm.unpermute(perm, dL, Ls, n)
    torch.cuda.synchronize()
    assert np.array_equal(Ls.cpu().numpy().view(np.uint32)[sample], ref_sample)
    m_c, c_c = out["caller"]
    m_s, c_s = out["spatial"]
    assert int(m_c.astype(np.uint64).sum()) == n
    assert np.array_equal(m_c, m_s)
    # the same labels: the FP64-merged sums of the two orders round to FP32 at
    # most one ulp apart
    assert np.all(np.abs(c_c - c_s) <= np.spacing(np.abs(c_c)))


def test_config3_full_size_sample_and_properties(ckm, oracle, cuda):
    """Config 3 at its size: n = 2^24, d = 128, k = 1024 (1024-component
    mixture, centres N(0, 4I), sigma log-U[0.25, 1], Dirichlet(1) weights),
    two tensor-core iterations (ckm_tc_fused_f32, fp16 operands) from the
    first-k centroids, the prepared set sorted by label after the first as
    the benchmark runs it.  Per iteration: the labels of a 16384-point sample
    equal the oracle's from the same input centroids, the masses equal the
    label counts, and the centroids of the non-empty clusters are within 1e-6
    (normwise relative) of the FP64 means of their points under the returned
    labels; the empty ones are NaN."""
    import torch
    n, d, k = 1 << 24, 128, 1024
    if not ckm.tc_supported(d, k):
        pytest.skip("tensor-core path not supported on this device")
    P = torch.empty(n * d, dtype=torch.float32, device=cuda)
    ckm.generate_mixture_ex(P, n, d, k, 42, center=("normal", 0.0, 2.0), sigma=("loguniform", 0.25, 1.0),
                            dirichlet=True)
    Pv = P.view(d, n)
    tcp = ckm.TensorCorePoints(P, n, d)
    C = [Pv[:, :k].reshape(-1).clone(), torch.empty(k * d, dtype=torch.float32, device=cuda)]
    L = torch.empty(n, dtype=torch.int32, device=cuda)
    M = torch.empty(k, dtype=torch.int32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    stats = torch.zeros(2, dtype=torch.int32, device=cuda)
    idx = np.sort(np.random.default_rng(11).choice(n, size=1 << 14, replace=False))
    Xs = np.ascontiguousarray(Pv[:, torch.from_numpy(idx).to(cuda)].cpu().numpy()).reshape(-1)
    for it in range(2):
        Cin = C[it % 2].cpu().numpy()
        ckm.tc_fused(P, tcp, C[it % 2], C[(it + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stats)
        torch.cuda.synchronize()
        assert int(stats[1].item()) == 0, "device wait ran out"
        lab = L.cpu().numpy().view(np.uint32)
        ref = oracle.label_f32(Xs, len(idx), d, k, Cin)
        assert np.array_equal(lab[idx], ref), "iteration %d: %d sample labels differ" % (
            it, int((lab[idx] != ref).sum()))
        counts = torch.bincount(L.long(), minlength=k)
        assert torch.equal(M.long(), counts)
        sums = torch.zeros(k, d, dtype=torch.float64, device=cuda)
        for s0 in range(0, n, 1 << 22):
            sums.index_add_(0, L[s0:s0 + (1 << 22)].long(), Pv[:, s0:s0 + (1 << 22)].t().double())
        full = counts > 0
        means = sums[full] / counts[full].double()[:, None]
        got = C[(it + 1) % 2].view(d, k).t().double()[full]
        rel = parity.rel_centroid_error(got.cpu().numpy(), means.cpu().numpy())
        assert rel <= 1e-6, "iteration %d: relative centroid error %.3g" % (it, rel)
        assert torch.isnan(C[(it + 1) % 2].view(d, k).t()[~full]).all()
        if it == 0:
            tcp.sort(k)


def test_config4_full_size_lockstep(ckm, oracle, cuda):
    """Batched jobs at their size: 4096 jobs (n log-U[2^10, 2^18], d from
    {2, 8, 32, 64}, k log-U[4, 256] with k <= n/16, each its own mixture of k
    blobs with centres U[-10, 10]^d and sigma 1, the first k points as initial
    centroids) in one batch, one step.  Every job: masses equal its label
    counts, centroids within 1e-5 (normwise relative) of the FP64 means of its
    labels, empty clusters NaN; every 64th job: labels equal the oracle's."""
    import torch
    rng = np.random.default_rng(1234)
    jobs = []
    for j in range(4096):
        n = int(round(np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 18)))))
        d = int(rng.choice([2, 8, 32, 64]))
        k = int(round(np.exp(rng.uniform(np.log(4), np.log(256)))))
        k = max(1, min(k, n // 16))
        P = torch.empty(n * d, dtype=torch.float32, device=cuda)
        ckm.generate_mixture(P, n, d, k, 1234 + j, sigma=(1.0, 1.0))
        C0 = P.view(d, n)[:, :k].reshape(-1).clone()
        jobs.append(dict(points=P, centroids=C0.clone(), init=C0,
                         labels=torch.empty(n, dtype=torch.int32, device=cuda),
                         masses=torch.empty(k, dtype=torch.int32, device=cuda), n=n, d=d, k=k))
    b = ckm.Batch(jobs)
    try:
        b.step()
        b.sync()
        torch.cuda.synchronize()
        worst = 0.0
        for i, j in enumerate(jobs):
            n, d, k = j["n"], j["d"], j["k"]
            L = j["labels"].long()
            counts = torch.bincount(L, minlength=k)
            assert torch.equal(j["masses"].long(), counts), (i, n, d, k)
            sums = torch.zeros(k, d, dtype=torch.float64, device=cuda)
            sums.index_add_(0, L, j["points"].view(d, n).t().double())
            full = counts > 0
            means = sums[full] / counts[full].double()[:, None]
            Ck = j["centroids"].view(d, k).t()
            worst = max(worst, parity.rel_centroid_error(Ck.double()[full].cpu().numpy(), means.cpu().numpy()))
            assert torch.isnan(Ck[~full]).all(), (i, n, d, k)
            if i % 64 == 0:
                ref = oracle.label_f32(j["points"].cpu().numpy(), n, d, k, j["init"].cpu().numpy())
                lab = j["labels"].cpu().numpy().view(np.uint32)
                assert np.array_equal(lab, ref), (i, n, d, k, int((lab != ref).sum()))
        assert worst <= 1e-5, worst
    finally:
        b.close()


def test_config2a_end_to_end_full_size(ckm, oracle, cuda):
    """The HBM-scale workload end to end at its size through the C ABI with
    host buffers: ckm_kmeans_run_f32 (single stage, 50 iterations, the
    spatial order taken automatically) over n = 2^28, d = 4, k = 16.  The
    returned masses equal the counts of the returned labels (which sum to n),
    the returned centroids are within 1e-5 (normwise relative) of the FP64
    means of the points under those labels, and on a 2^20-point sample the
    labels equal the oracle's from the centroids the last iteration started
    from (taken from a 49-iteration run; every mismatch adjudicated in FP64
    against the derived near-tie bound)."""
    import torch
    n, d, k, iters = 1 << 28, 4, 16, 50
    dP = _c2a(ckm, cuda, n)
    P = dP.cpu().numpy()
    C0 = dP.view(d, n)[:, :k].reshape(-1).cpu().numpy()
    C, M, L, info = ckm.kmeans_run(P, d, k, iters, C0, pipeline="single_stage")
    assert info.iterations == iters
    dL = torch.from_numpy(L.view(np.int32)).to(cuda).long()
    counts = torch.bincount(dL, minlength=k)
    assert int(counts.sum().item()) == n
    assert np.array_equal(M.astype(np.int64), counts.cpu().numpy())
    sums = torch.zeros(k, d, dtype=torch.float64, device=cuda)
    Pv = dP.view(d, n)
    for s0 in range(0, n, 1 << 24):
        sums.index_add_(0, dL[s0:s0 + (1 << 24)], Pv[:, s0:s0 + (1 << 24)].t().double())
    full = (counts > 0).cpu().numpy()
    means = (sums / counts.clamp(min=1).double()[:, None]).cpu().numpy()
    got = C.reshape(d, k).T.astype(np.float64)
    assert parity.rel_centroid_error(got[full], means[full]) <= 1e-5
    del dL, sums
    # the last iteration's labels on a sample, from a 49-iteration run's centroids
    C49 = ckm.kmeans_run(P, d, k, iters - 1, C0, pipeline="single_stage")[0]
    idx = np.sort(np.random.default_rng(5).choice(n, size=1 << 20, replace=False))
    Xs = np.ascontiguousarray(P.reshape(d, n)[:, idx]).reshape(-1)
    ref = oracle.label_f32(Xs, len(idx), d, k, C49)
    got_l = L.view(np.uint32)[idx]
    if np.any(got_l != ref):
        parity.adjudicate(Xs, len(idx), d, k, got_l, ref, C49, C49, prev_slack_ulps=1)
