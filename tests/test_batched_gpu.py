"""Batched jobs (ckm_batch_*): many independent k-means problems of uneven
n, d and k advanced by one persistent launch per iteration.  Every job must
behave exactly like the same job run alone: per iteration (lockstep), each
job's labels are bit-exact against the oracle's FP32 labeling with that
iteration's input centroids, masses are exact, centroids are within the
fused tests' tolerance of the FP64 means."""
import numpy as np
import pytest

from conftest import blobs
from test_fused_gpu import check_centroids

pytestmark = pytest.mark.gpu


def make_jobs(cuda, oracle, shapes, seed=0):
    import torch
    jobs, host = [], []
    for i, (n, d, k) in enumerate(shapes):
        P = blobs(n, d, max(1, min(k, 32)), seed=seed * 1000 + i)
        C = oracle.first_x_f32(P, n, d, k)
        jobs.append(dict(points=torch.from_numpy(P).to(cuda), centroids=torch.from_numpy(C).to(cuda),
                         labels=torch.zeros(max(n, 1), dtype=torch.int32, device=cuda),
                         masses=torch.zeros(k, dtype=torch.int32, device=cuda), n=n, d=d, k=k))
        host.append(P)
    return jobs, host


SHAPES = [(1024, 2, 4), (5000, 8, 37), (777, 3, 9), (20000, 32, 64), (3000, 64, 256), (65536, 4, 16),
          (1031, 5, 7), (100, 16, 6), (12345, 2, 200), (40000, 8, 8), (2048, 64, 64), (1, 2, 1)]


@pytest.mark.parametrize("opts", [dict(), dict(tile_points=256, ctas_per_sm=2), dict(tile_points=4096),
                                  dict(autotune=True)])
def test_batch_lockstep_matches_oracle(ckm, oracle, cuda, opts):
    import torch
    jobs, host = make_jobs(cuda, oracle, SHAPES, seed=1)
    b = ckm.Batch(jobs, **opts)
    try:
        for it in range(4):
            b.sync()
            torch.cuda.synchronize()
            Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
            b.step()
            b.sync()
            torch.cuda.synchronize()
            for j, P, C0 in zip(jobs, host, Cin):
                n, d, k = j["n"], j["d"], j["k"]
                lab = j["labels"][:n].cpu().numpy().view(np.uint32)
                ref = oracle.label_f32(P, n, d, k, C0)
                assert np.array_equal(lab, ref), (it, n, d, k, int((lab != ref).sum()))
                assert np.array_equal(j["masses"].cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
                check_centroids(oracle, P, n, d, k, ref, j["centroids"].cpu().numpy())
        sh, its = b.status()
        assert np.all(its == 4)
    finally:
        b.close()


def test_batch_graph_run_equals_steps(ckm, oracle, cuda):
    import torch
    jobsA, host = make_jobs(cuda, oracle, SHAPES, seed=2)
    jobsB, _ = make_jobs(cuda, oracle, SHAPES, seed=2)
    a = ckm.Batch(jobsA, tile_points=1024, ctas_per_sm=1)
    b = ckm.Batch(jobsB, tile_points=1024, ctas_per_sm=1)
    try:
        a.run(6, use_graph=True)
        for _ in range(6):
            b.step()
        b.sync()
        torch.cuda.synchronize()
        for ja, jb, P in zip(jobsA, jobsB, host):
            ca, cb = ja["centroids"].cpu().numpy(), jb["centroids"].cpu().numpy()
            nan = np.isnan(ca)
            assert np.array_equal(nan, np.isnan(cb))
            assert np.allclose(ca[~nan], cb[~nan], rtol=1e-5, atol=1e-4)
        assert np.all(a.status()[1] == 6)
        # replaying the cached graph continues from the current state
        a.run(6, use_graph=True)
        torch.cuda.synchronize()
        assert np.all(a.status()[1] == 12)
    finally:
        a.close()
        b.close()


def test_batch_inactive_jobs_are_skipped_and_shift_reported(ckm, oracle, cuda):
    import torch
    jobs, host = make_jobs(cuda, oracle, SHAPES[:6], seed=3)
    b = ckm.Batch(jobs)
    try:
        active = [1, 0, 1, 0, 1, 1]
        b.set_active(active)
        before = [j["centroids"].cpu().numpy().copy() for j in jobs]
        b.step()
        b.sync()
        torch.cuda.synchronize()
        sh, its = b.status()
        for i, (j, a, C0) in enumerate(zip(jobs, active, before)):
            C1 = j["centroids"].cpu().numpy()
            if not a:
                assert its[i] == 0 and np.array_equal(C1, C0)
            else:
                assert its[i] == 1
                ok = ~np.isnan(C1)
                want = np.abs(C1[ok] - C0[ok]).max() / max(np.abs(C0).max(), 1e-30)
                assert abs(sh[i] - want) <= 1e-6 * max(1.0, want)
    finally:
        b.close()


def test_batch_rejects_bad_jobs(ckm, cuda):
    import torch
    t = torch.zeros(16, dtype=torch.float32, device=cuda)
    with pytest.raises(ckm.CkmError):
        ckm.Batch([dict(points=t, centroids=t, labels=t, masses=t, n=4, d=0, k=2)])
    with pytest.raises(ckm.CkmError):
        ckm.Batch([])


def test_batch_convergence_stop(ckm, oracle, cuda):
    """tolerance / max_iterations: every job parks itself after the first
    iteration whose relative centroid shift is below the tolerance (or after
    max_iterations), exactly as if it had run alone with that stopping rule;
    later steps leave it untouched."""
    import torch
    from test_pipelines_gpu import _e2e_check
    shapes = [(4000, 2, 4), (6000, 8, 12), (3000, 3, 5), (8000, 16, 20), (2000, 32, 16), (5000, 4, 6)]
    jobs, host = make_jobs(cuda, oracle, shapes, seed=7)
    init = [oracle.first_x_f32(P, j["n"], j["d"], j["k"]) for j, P in zip(jobs, host)]
    b = ckm.Batch(jobs, tolerance=1e-4, max_iterations=25)
    try:
        for _ in range(40):
            b.step()
        b.sync()
        torch.cuda.synchronize()
        sh, its = b.status()
        assert np.all(its >= 1) and np.all(its <= 25)
        assert np.any(its < 25), "some jobs converge before the cap"
        for i, (j, P, C0) in enumerate(zip(jobs, host, init)):
            n, d, k = j["n"], j["d"], j["k"]
            if its[i] < 25:
                assert sh[i] < 1e-4
            C = j["centroids"].cpu().numpy()
            L = j["labels"][:n].cpu().numpy().view(np.uint32)
            M = j["masses"].cpu().numpy().view(np.uint32)
            it = int(its[i])
            _e2e_check(oracle, P, n, d, k, it, C0, C, M, L,
                       lambda: ckm.kmeans_run(P, d, k, it - 1, C0)[0], prev_slack_ulps=2)
    finally:
        b.close()


def test_batch_screened_labels_ties_and_nan(ckm, oracle, cuda):
    """Duplicated centroids (exact ties: the lowest index must win) and a NaN
    centroid (an empty cluster: never chosen) in jobs of d = 8..64: labels
    must stay the oracle's."""
    import torch
    # SIMT screen: d = 8, 16, (32, k < 64), (64, k < 32); tensor-core screen:
    # (32, k >= 64), (64, k >= 32)
    shapes = [(6000, 8, 24), (5000, 32, 40), (3000, 64, 17), (4000, 16, 64), (4000, 64, 40), (3000, 32, 70)]
    jobs, host = make_jobs(cuda, oracle, shapes, seed=11)
    for j in jobs:
        d, k = j["d"], j["k"]
        C = j["centroids"].cpu().numpy().reshape(d, k)
        C[:, 7] = C[:, 3]        # exact duplicate
        C[:, k - 1] = C[:, 5]    # duplicate with the higher index last
        C[:, 10] = np.nan        # empty cluster
        j["centroids"].copy_(torch.from_numpy(np.ascontiguousarray(C).reshape(-1)))
    b = ckm.Batch(jobs)
    try:
        for it in range(2):
            b.sync()
            torch.cuda.synchronize()
            Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
            b.step()
            b.sync()
            torch.cuda.synchronize()
            for j, P, C0 in zip(jobs, host, Cin):
                n, d, k = j["n"], j["d"], j["k"]
                lab = j["labels"][:n].cpu().numpy().view(np.uint32)
                ref = oracle.label_f32(P, n, d, k, C0)
                assert np.array_equal(lab, ref), (it, n, d, k, int((lab != ref).sum()))
                if it == 0:
                    assert not np.any(lab == 7) and not np.any(lab == 10) and not np.any(lab == k - 1)
                assert np.array_equal(j["masses"].cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
                check_centroids(oracle, P, n, d, k, ref, j["centroids"].cpu().numpy())
    finally:
        b.close()


def test_batch_screen_fallback_offsets_and_huge_centroids(ckm, oracle, cuda):
    """Jobs of d = 8..64 (FP32 screen; tensor-core screen for d = 32 with
    k >= 64 and d = 64 with k >= 32) whose points sit far from the origin
    (many points fall back from the screen to the exact loop) or that hold a
    huge or an infinite centroid (every point falls back): labels stay the
    oracle's."""
    import torch
    # (n, d, k, change)
    cases = [(5000, 8, 20, "offset"), (4000, 64, 24, "offset"), (6000, 32, 30, "offset"), (3000, 64, 9, "huge"),
             (3000, 64, 40, "inf"), (2000, 32, 5, "-huge"), (2500, 64, 33, "huge"), (2600, 32, 48, "inf"),
             (4000, 64, 48, "offset"), (5000, 32, 80, "offset"), (2600, 32, 72, "inf"), (2200, 32, 66, "huge")]
    jobs, host = make_jobs(cuda, oracle, [c[:3] for c in cases], seed=13)
    for i, (j, (n, d, k, change)) in enumerate(zip(jobs, cases)):
        if change == "offset":
            host[i] = (host[i] + np.float32(2500.0)).astype(np.float32)
            j["points"].copy_(torch.from_numpy(host[i]))
            C = oracle.first_x_f32(host[i], n, d, k).reshape(d, k)
        else:
            C = j["centroids"].cpu().numpy().reshape(d, k)
            if change == "huge":
                C[:, 2] = 1e30
            elif change == "-huge":
                C[:, 1] = -1e31
            else:
                C[1, 3] = np.inf
        j["centroids"].copy_(torch.from_numpy(np.ascontiguousarray(C).reshape(-1)))
    b = ckm.Batch(jobs)
    try:
        Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
        b.step()
        b.sync()
        torch.cuda.synchronize()
        for j, P, C0 in zip(jobs, host, Cin):
            n, d, k = j["n"], j["d"], j["k"]
            lab = j["labels"][:n].cpu().numpy().view(np.uint32)
            ref = oracle.label_f32(P, n, d, k, C0)
            assert np.array_equal(lab, ref), (n, d, k, int((lab != ref).sum()))
            assert np.array_equal(j["masses"].cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
    finally:
        b.close()


UMMA_SHAPES = [(20000, 32, 16), (4099, 64, 17), (1000, 32, 31), (129, 64, 63), (128, 32, 64), (3000, 64, 65),
               (5000, 32, 100), (2500, 64, 128), (100, 32, 200), (4500, 64, 255), (3333, 32, 256), (1, 64, 16),
               (777, 64, 256), (9000, 32, 20)]


@pytest.mark.parametrize("umma", ["1", "0"])
def test_batch_tensor_core_path_lockstep(ckm, oracle, cuda, umma, monkeypatch):
    """d = 32 / 64 jobs with 16 <= k <= 256 take the tcgen05 path in
    512-thread CTAs (CKM_BATCH_UMMA=0 switches it off): k not a multiple of
    the column groups, n not a multiple of 128 and below 128.  Labels stay the
    oracle's bit for bit on both paths."""
    import torch
    monkeypatch.setenv("CKM_BATCH_UMMA", umma)
    jobs, host = make_jobs(cuda, oracle, UMMA_SHAPES, seed=21)
    b = ckm.Batch(jobs, tile_points=1024, ctas_per_sm=1)
    try:
        for it in range(3):
            b.sync()
            torch.cuda.synchronize()
            Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
            b.step()
            b.sync()
            torch.cuda.synchronize()
            for j, P, C0 in zip(jobs, host, Cin):
                n, d, k = j["n"], j["d"], j["k"]
                lab = j["labels"][:n].cpu().numpy().view(np.uint32)
                ref = oracle.label_f32(P, n, d, k, C0)
                assert np.array_equal(lab, ref), (it, n, d, k, int((lab != ref).sum()))
                assert np.array_equal(j["masses"].cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
                check_centroids(oracle, P, n, d, k, ref, j["centroids"].cpu().numpy())
        assert np.all(b.status()[1] == 3)
    finally:
        b.close()


def test_batch_tensor_core_path_edge_values(ckm, oracle, cuda):
    """On the tcgen05 path: exact ties, a NaN centroid, points with NaN or
    infinite coordinates, points beyond fp16's range (|x| >= 2^15: the full
    exact scan), points far from every centroid (many candidates) and
    duplicated points.  Labels stay the oracle's."""
    import torch
    shapes = [(6000, 32, 40), (5000, 64, 64), (3000, 64, 200), (4000, 32, 17)]
    jobs, host = make_jobs(cuda, oracle, shapes, seed=23)
    for i, j in enumerate(jobs):
        n, d, k = j["n"], j["d"], j["k"]
        P = host[i].reshape(d, n).copy()
        P[:, 50:400] = P[:, 50:51]              # duplicates
        P[3, 500] = np.nan
        P[0, 600] = np.inf
        P[1, 700] = -np.inf
        P[:, 800:900] += np.float32(40000.0)     # |x| >= 2^15
        P[2, 950] = np.float32(70000.0)          # beyond fp16's largest finite value
        P[:, 1000:1100] *= np.float32(300.0)     # far from every centroid
        host[i] = np.ascontiguousarray(P).reshape(-1)
        j["points"].copy_(torch.from_numpy(host[i]))
        C = np.nan_to_num(oracle.first_x_f32(host[i], n, d, k), nan=0.0, posinf=1.0, neginf=-1.0).reshape(d, k)
        C = np.clip(C, -100.0, 100.0)
        C[:, 7] = C[:, 3]
        C[:, k - 1] = C[:, 5]
        C[:, 10] = np.nan
        j["centroids"].copy_(torch.from_numpy(np.ascontiguousarray(C, dtype=np.float32).reshape(-1)))
    b = ckm.Batch(jobs, tile_points=1024, ctas_per_sm=1)
    try:
        Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
        b.step()
        b.sync()
        torch.cuda.synchronize()
        for j, P, C0 in zip(jobs, host, Cin):
            n, d, k = j["n"], j["d"], j["k"]
            lab = j["labels"][:n].cpu().numpy().view(np.uint32)
            ref = oracle.label_f32(P, n, d, k, C0)
            assert np.array_equal(lab, ref), (n, d, k, int((lab != ref).sum()), np.nonzero(lab != ref)[0][:10])
            assert not np.any(lab == 7) and not np.any(lab == 10) and not np.any(lab == k - 1)
            assert np.array_equal(j["masses"].cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k))
    finally:
        b.close()


def test_batch_tensor_core_wait_timeout_is_reported(ckm, oracle, cuda, monkeypatch):
    """Failure detection without a GPU fault: with CKM_BATCH_TEST_STALL=1 the
    first half of every CTA issues no MMA, so its bounded wait for the tensor
    cores finds nothing and runs out (1 ms).  The CTA frees its tensor memory
    and stops, the job is parked with the failed bit, ckm_batch_status
    reports CKM_ERR_CUDA, and the context stays usable: a new batch afterwards
    matches the oracle."""
    import torch
    monkeypatch.setenv("CKM_BATCH_TEST_STALL", "1")
    jobs, _ = make_jobs(cuda, oracle, [(20000, 64, 64), (9000, 32, 40), (3000, 8, 10)], seed=31)
    b = ckm.Batch(jobs, tile_points=1024, ctas_per_sm=1)
    try:
        b.step()
        torch.cuda.synchronize()
        with pytest.raises(ckm.CkmError) as e:
            b.status()
        assert "tensor cores" in str(e.value)
        assert e.value.status == -7  # CKM_ERR_TIMEOUT
    finally:
        b.close()
    monkeypatch.delenv("CKM_BATCH_TEST_STALL")
    jobs, host = make_jobs(cuda, oracle, [(20000, 64, 64), (9000, 32, 40)], seed=32)
    b = ckm.Batch(jobs, tile_points=1024, ctas_per_sm=1)
    try:
        Cin = [j["centroids"].cpu().numpy().copy() for j in jobs]
        b.step()
        b.sync()
        torch.cuda.synchronize()
        for j, P, C0 in zip(jobs, host, Cin):
            n, d, k = j["n"], j["d"], j["k"]
            ref = oracle.label_f32(P, n, d, k, C0)
            assert np.array_equal(j["labels"][:n].cpu().numpy().view(np.uint32), ref)
        b.status()
    finally:
        b.close()
