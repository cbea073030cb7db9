"""Serving loop (ckm_server_*): jobs submitted with host arrays, admitted
within a device budget, advanced in batched rounds or in the large-job lane,
each retired at its own stopping iteration (relative centroid shift below the
tolerance, or the cap).  Every result must be what the same job gives when
run alone for that many iterations: labels equal to the oracle's FP32
KmeansNaive run except at FP64 near-ties, masses exact, centroids within the
fused tolerance of the FP64 means of the labels."""
import numpy as np
import pytest

import parity
from conftest import blobs
from test_pipelines_gpu import _e2e_check

pytestmark = pytest.mark.gpu


def _jobs(oracle, shapes, seed):
    out = []
    for i, (n, d, k) in enumerate(shapes):
        P = blobs(n, d, max(1, min(k, 24)), seed=seed * 100 + i, spread=6.0, sigma=0.8)
        C0 = oracle.first_x_f32(P, n, d, k)
        out.append((P, C0, n, d, k))
    return out


def _check(ckm, oracle, job, res, tol, cap):
    P, C0, n, d, k = job
    assert res["status"] == 0
    its = res["iterations"]
    assert 1 <= its <= cap
    if res["converged"]:
        assert res["shift"] < tol
    else:
        assert its == cap
    _e2e_check(oracle, P, n, d, k, its, C0, res["centroids"], res["masses"], res["labels"],
               lambda: ckm.kmeans_run(P, d, k, its - 1, C0)[0], prev_slack_ulps=2)


def test_server_batched_lane_matches_single_runs(ckm, oracle, cuda):
    shapes = [(3000, 2, 4), (5000, 8, 12), (1200, 3, 5), (8000, 16, 20), (2500, 32, 16), (6000, 4, 6),
              (4096, 64, 8), (777, 2, 3), (10000, 8, 40), (1500, 5, 7)] * 3
    jobs = _jobs(oracle, shapes, seed=1)
    tol, cap = 1e-4, 20
    S = ckm.Server(tolerance=tol, max_iterations=cap, round_iterations=3)
    try:
        for t, (P, C0, n, d, k) in enumerate(jobs):
            S.submit(P, C0, n, d, k, tag=t)
        S.drain()
        res = S.poll()
        assert sorted(r["tag"] for r in res) == list(range(len(jobs)))
        assert all(r["lane"] == 0 for r in res)
        assert any(r["converged"] for r in res)
        for r in res:
            _check(ckm, oracle, jobs[r["tag"]], r, tol, cap)
    finally:
        S.close()


def test_server_continuous_batching(ckm, oracle, cuda):
    """Jobs that arrive while rounds are on the GPU join a later round and run
    beside the jobs already there, and each result is the same as the job's
    run alone.

    The first wave is long-running work (uniform points, no cluster
    structure, so Lloyd creeps on for the whole 50-iteration cap at one
    iteration per round); it is checked for completion only.  The second wave
    arrives once two rounds have run; its jobs are Gaussian blobs started from
    their blob centres, so no point sits near a tie and the run alone must
    give the same labels and masses exactly and centroids within 1e-5
    relative, and the oracle's run of the same length agrees as well."""
    import time
    tol, cap = 1e-6, 50

    def uniform_job(n, d, k, seed):
        P = np.ascontiguousarray(np.random.default_rng(seed).uniform(-5, 5, size=(d, n)).astype(np.float32)).reshape(-1)
        return P, oracle.first_x_f32(P, n, d, k), n, d, k

    def blob_job(n, d, k, seed):
        rng = np.random.default_rng(seed)
        centres = rng.uniform(-10, 10, size=(k, d))
        X = centres[rng.integers(0, k, size=n)] + rng.standard_normal((n, d))
        P = np.ascontiguousarray(X.astype(np.float32).T).reshape(-1)
        C0 = np.ascontiguousarray((centres + 0.1 * rng.standard_normal((k, d))).astype(np.float32).T).reshape(-1)
        return P, C0, n, d, k

    rng = np.random.default_rng(4)
    wave1 = [uniform_job(1 << 17, 32, 64, 100 + i) for i in range(12)]
    wave2 = [blob_job(int(rng.integers(2000, 20000)), int(rng.choice([2, 4, 16])), int(rng.integers(3, 12)), 200 + i)
             for i in range(12)]
    S = ckm.Server(tolerance=tol, max_iterations=cap, round_iterations=1)
    try:
        for t, (P, C0, n, d, k) in enumerate(wave1):
            S.submit(P, C0, n, d, k, tag=t)
        t0 = time.perf_counter()
        while S.stats()["rounds"] < 2:
            assert time.perf_counter() - t0 < 30, "the server ran no round"
            time.sleep(0.0005)
        rounds_at_submit = S.stats()["rounds"]
        for t, (P, C0, n, d, k) in enumerate(wave2):
            S.submit(P, C0, n, d, k, tag=100 + t)
        S.drain()
        res = {r["tag"]: r for r in S.poll()}
        assert sorted(res) == list(range(len(wave1))) + [100 + t for t in range(len(wave2))]
        assert all(r["status"] == 0 and r["lane"] == 0 for r in res.values())
        first2 = min(res[100 + t]["first_round"] for t in range(len(wave2)))
        # the late jobs joined rounds after those already launched ...
        assert all(res[100 + t]["first_round"] > rounds_at_submit for t in range(len(wave2)))
        assert all(res[t]["first_round"] >= 1 for t in range(len(wave1)))
        # ... while jobs of the first wave were still running beside them
        assert max(res[t]["last_round"] for t in range(len(wave1))) >= first2
        for t, job in enumerate(wave2):
            r = res[100 + t]
            _check(ckm, oracle, job, r, tol, cap)
            P, C0, n, d, k = job
            Ca, Ma, La, _ = ckm.kmeans_run(P, d, k, r["iterations"], C0)
            assert np.array_equal(La.view(np.uint32), r["labels"])
            assert np.array_equal(Ma, r["masses"])
            assert parity.rel_centroid_error(r["centroids"], Ca) <= 1e-5
    finally:
        S.close()


def test_server_large_lane(ckm, oracle, cuda):
    """Jobs at or above large_work run alone: on the tensor cores when d >= 32
    (lane 1), else on the SIMT fused kernel (lane 2); small ones in between
    keep flowing through the batched lane."""
    shapes = [(20000, 64, 32), (30000, 4, 16), (2000, 8, 6), (3000, 2, 5)]
    jobs = _jobs(oracle, shapes, seed=2)
    tol, cap = 1e-4, 15
    S = ckm.Server(tolerance=tol, max_iterations=cap, large_work=1 << 20)
    try:
        for t, (P, C0, n, d, k) in enumerate(jobs):
            S.submit(P, C0, n, d, k, tag=t)
        S.drain()
        res = {r["tag"]: r for r in S.poll()}
        want_tc = 1 if ckm.tc_supported(64, 32) else 2
        assert res[0]["lane"] == want_tc and res[1]["lane"] == 2
        assert res[2]["lane"] == 0 and res[3]["lane"] == 0
        for t, r in res.items():
            _check(ckm, oracle, jobs[t], r, tol, cap)
    finally:
        S.close()


def test_server_budget_and_bad_jobs(ckm, cuda):
    """A job larger than the whole budget, or with no points, is refused at
    submit; jobs that fit only one at a time still all complete."""
    S = ckm.Server(device_budget_bytes=1 << 20, max_iterations=5)
    try:
        big = np.zeros(4 * 200000, np.float32)
        with pytest.raises(ckm.CkmError) as e:
            S.submit(big, big[:16], 200000, 4, 4, tag=1)
        assert e.value.status == -10
        with pytest.raises(ckm.CkmError):
            S.submit(big[:0], big[:16], 0, 4, 4, tag=2)
        P = blobs(20000, 4, 4, seed=3)
        for t in range(6):   # each ~0.4 MiB: at most two admitted at a time
            S.submit(P, P.reshape(4, -1)[:, :4].copy().reshape(-1), 20000, 4, 4, tag=10 + t)
        S.drain()
        res = S.poll()
        assert sorted(r["tag"] for r in res) == list(range(10, 16))
        assert all(r["status"] == 0 for r in res)
    finally:
        S.close()
