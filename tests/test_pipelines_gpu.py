"""Three-stage functors and the host-level pipelines (ckm_kmeans_run_*),
each against the oracle.

The three-stage functors follow the reference contracts: labeling writes
labels (labeling_factory.hpp:33-48); mass update adds counts into masses
(mass_update_factory.hpp:36-48); centroid update adds per-label sums into the
zero-filled centroids (centroid_update_factory.hpp:37-54); divide is
MatrixBinaryOp::row (matrix_binary_op.cl:98-114).  The pipelines are
AbstractKmeans::operator() for the four `kmeans.pipeline` names
(bench.cpp:319-404) with host arrays.
"""
import numpy as np
import pytest

import parity
from conftest import blobs
from test_fused_gpu import check_centroids, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,d,k", [(40000, 4, 16), (9999, 3, 5), (5000, 24, 30), (20000, 2, 300)])
def test_three_stage_functors(ckm, oracle, cuda, n, d, k):
    import torch
    P = blobs(n, d, k, seed=n + d)
    C = oracle.first_x_f32(P, n, d, k)
    dP, dC = to_dev(P, cuda), to_dev(C, cuda)
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    ckm.labeling(dP, dC, dL, n, d, k)
    torch.cuda.synchronize()
    ref = oracle.label_f32(P, n, d, k, C)
    assert np.array_equal(dL.cpu().numpy().view(np.uint32), ref)

    dM = torch.full((k,), 5, dtype=torch.int32, device=cuda)
    ckm.mass_update(dL, dM, n, k)
    torch.cuda.synchronize()
    assert np.array_equal(dM.cpu().numpy().view(np.uint32), oracle.mass_u32(ref, k) + 5)

    dS = torch.zeros(k * d, dtype=torch.float32, device=cuda)
    S = ckm.new_scratch(d, k, cuda)
    ckm.centroid_update(dP, dS, dL, dM, S, n, d, k, ckm.MODE_ACCUMULATE)
    torch.cuda.synchronize()
    sums, masses = oracle.sums_f64(P, n, d, k, ref)
    assert np.allclose(dS.cpu().numpy(), sums, rtol=2e-6, atol=2e-6 * np.abs(P).max() * 10)

    dM2 = torch.from_numpy(masses.astype(np.uint32).view(np.int32)).to(cuda)
    ckm.divide_row(dS, dM2, d, k)
    torch.cuda.synchronize()
    check_centroids(oracle, P, n, d, k, ref, dS.cpu().numpy())


@pytest.mark.parametrize("kind", ["f32", "f64", "u32", "u64"])
def test_matrix_add_accumulates(ckm, cuda, kind):
    """ckm_matrix_add_*: a += b elementwise (MatrixBinaryOp::matrix Add,
    matrix_binary_op.hpp:149-188), the buffered strategies' accumulation of
    per-chunk sums and masses; the integer forms wrap mod 2^32 / 2^64."""
    import ctypes
    import torch
    rng = np.random.default_rng(11)
    count = 100003
    dt = {"f32": np.float32, "f64": np.float64, "u32": np.uint32, "u64": np.uint64}[kind]
    if kind.startswith("f"):
        a = rng.normal(size=count).astype(dt)
        b = rng.normal(size=count).astype(dt)
        want = a + b
    else:
        hi = 1 << (32 if kind == "u32" else 63)
        a = rng.integers(0, hi, size=count, dtype=np.uint64).astype(dt)
        b = rng.integers(0, hi, size=count, dtype=np.uint64).astype(dt)
        want = a + b                       # numpy wraps like the device
    view = {"u32": np.int32, "u64": np.int64}.get(kind, dt)
    da = torch.from_numpy(a.view(view).copy()).to(cuda)
    db = torch.from_numpy(b.view(view).copy()).to(cuda)
    fn = getattr(ckm.lib(), "ckm_matrix_add_" + kind)
    fn.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    s = torch.cuda.current_stream()
    assert fn(count, da.data_ptr(), db.data_ptr(), s.cuda_stream) == 0
    torch.cuda.synchronize()
    got = da.cpu().numpy().view(dt)
    assert np.array_equal(got, want)
    assert fn(0, da.data_ptr(), db.data_ptr(), s.cuda_stream) == 0   # empty: no work, no error


def test_mass_update_exact_uniform_labels(ckm, cuda):
    """The reference's histogram test (test/histogram.cpp:31-39, 211-226):
    exact counts of 1 Mi uniform labels for 2..16 bins."""
    import torch
    rng = np.random.default_rng(3)
    n = 1 << 20
    for k in (2, 4, 8, 16):
        labels = rng.integers(0, k, size=n).astype(np.uint32)
        dL = to_dev(labels.view(np.int32), cuda)
        dM = torch.zeros(k, dtype=torch.int32, device=cuda)
        ckm.mass_update(dL, dM, n, k)
        torch.cuda.synchronize()
        assert np.array_equal(dM.cpu().numpy().view(np.uint32), np.bincount(labels, minlength=k))


@pytest.mark.parametrize("rows,cols,kind", [(4, 256, "ascending"), (4, 256, "large"), (4, 256, "random"),
                                            (4, 65536, "random"), (2048, 65536, "random"),
                                            (256, 46080, "random"), (4, 57344, "random")])
def test_reduce_vector_parcol_exact(ckm, cuda, rows, cols, kind):
    """The reference's ReduceVectorParcol shapes (test/reduce_vector.cpp:74-221),
    uint32 column sums wrapping mod 2^32."""
    import torch
    rng = np.random.default_rng(rows * cols)
    if kind == "ascending":
        data = np.arange(rows * cols, dtype=np.uint32)
    elif kind == "large":
        data = np.full(rows * cols, 1 << 31, dtype=np.uint32)
    else:
        data = rng.integers(0, 1 << 32, size=rows * cols, dtype=np.uint64).astype(np.uint32)
    want = data.reshape(cols, rows).astype(np.uint64).sum(axis=0) % (1 << 32)
    dD = to_dev(data.view(np.int32), cuda)
    ckm.reduce_vector_parcol(dD, cols, rows)
    torch.cuda.synchronize()
    assert np.array_equal(dD[:rows].cpu().numpy().view(np.uint32), want.astype(np.uint32))


def _e2e_check(oracle, P, n, d, k, iters, C0, C, M, L, ours_prev=None, prev_slack_ulps=0):
    """End-to-end against the oracle's FP32 KmeansNaive restatement: every
    label mismatch is adjudicated in FP64 against the derived near-tie bound
    (tests/parity.py: the FP32 distance rounding (d + 4) 2^-24 plus the
    measured drift between the two runs' last input centroids, which
    `ours_prev()` supplies: our centroids after iters - 1 iterations); masses
    equal the counts of our labels; centroids are the FP64 means of our
    labels.  A job that ran on another path (batched, served) passes a rerun
    of itself alone as `ours_prev`, with prev_slack_ulps = 2 for the rounding
    of the two paths' FP64 merges."""
    Cr, Mr, Lr = oracle.lloyd_f32(P, n, d, k, iters, C0)
    if np.any(L != Lr):
        assert ours_prev is not None, "label mismatches and no way to rerun our side"
        Cref_prev, _, _ = oracle.lloyd_f32(P, n, d, k, iters - 1, C0)
        parity.adjudicate(P, n, d, k, L, Lr, ours_prev(), Cref_prev, prev_slack_ulps)
    assert np.array_equal(M, oracle.mass_u32(L, k))
    check_centroids(oracle, P, n, d, k, L, C)


@pytest.mark.parametrize("pipeline", ["single_stage", "three_stage", "single_stage_buffered",
                                      "three_stage_buffered"])
def test_pipelines_end_to_end(ckm, oracle, cuda, pipeline):
    n, d, k, iters = 100003, 4, 10, 12
    P = blobs(n, d, k, seed=99)
    C0 = oracle.first_x_f32(P, n, d, k)
    extra = {}
    if pipeline.endswith("buffered"):
        # force streaming: 5 chunks of 24k points; the budget holds the 3
        # streaming slots plus 2 resident chunks (+ the fixed 1 MiB reserve)
        extra = dict(chunk_bytes=24000 * d * 4, device_budget_bytes=(24000 * (d + 1) * 4) * 5 + (1 << 20) + 65536)
    C, M, L, info = ckm.kmeans_run(P, d, k, iters, C0, pipeline=pipeline, **extra)
    assert info.iterations == iters and info.kernel_launches > 0
    _e2e_check(oracle, P, n, d, k, iters, C0, C, M, L,
               lambda: ckm.kmeans_run(P, d, k, iters - 1, C0, pipeline=pipeline, **extra)[0])


@pytest.mark.parametrize("n,d,k,iters,mode", [(100003, 4, 10, 12, 1), (1 << 20, 4, 16, 10, 0), (60000, 2, 7, 9, 1),
                                              (50001, 8, 32, 8, 1), (40000, 3, 40, 6, 1)])
def test_single_stage_spatial_order(ckm, oracle, cuda, n, d, k, iters, mode):
    """single_stage with spatial_order = 1 (whenever the shape allows) or
    0 (auto: n >= 2^20): the iterations run on a sorted copy with box pruning
    and the labels come back in the caller's order; results as the oracle's.
    k = 40 is outside the pruned shapes and runs the caller's order."""
    P = blobs(n, d, k, seed=n + k)
    C0 = oracle.first_x_f32(P, n, d, k)
    C, M, L, info = ckm.kmeans_run(P, d, k, iters, C0, pipeline="single_stage", spatial_order=mode)
    assert info.iterations == iters
    _e2e_check(oracle, P, n, d, k, iters, C0, C, M, L.view(np.uint32),
               lambda: ckm.kmeans_run(P, d, k, iters - 1, C0, pipeline="single_stage", spatial_order=mode)[0])


@pytest.mark.parametrize("n,d,k,iters,mode", [(100003, 4, 10, 10, 1), (1 << 20, 4, 16, 9, 0), (50001, 8, 32, 8, 1)])
def test_three_stage_spatial_order(ckm, oracle, cuda, n, d, k, iters, mode):
    """three_stage with the spatial order: box-pruned labeling and the
    centroid update on the sorted copy, last iteration in the caller's
    order; results as the oracle's."""
    P = blobs(n, d, k, seed=3 * n + k)
    C0 = oracle.first_x_f32(P, n, d, k)
    C, M, L, info = ckm.kmeans_run(P, d, k, iters, C0, pipeline="three_stage", spatial_order=mode)
    assert info.iterations == iters
    _e2e_check(oracle, P, n, d, k, iters, C0, C, M, L.view(np.uint32),
               lambda: ckm.kmeans_run(P, d, k, iters - 1, C0, pipeline="three_stage", spatial_order=mode)[0])


@pytest.mark.parametrize("pipeline", ["single_stage", "three_stage"])
def test_spatial_order_converging(ckm, oracle, cuda, pipeline):
    """A spatial-order run that stops on the convergence test before the
    iteration cap ends on the sorted set; its labels are mapped back to the
    caller's order and equal the oracle's for that many iterations."""
    n, d, k = 100003, 4, 10
    P = blobs(n, d, k, seed=5)
    C0 = oracle.first_x_f32(P, n, d, k)
    C, M, L, info = ckm.kmeans_run(P, d, k, 60, C0, pipeline=pipeline, spatial_order=1, converge=True,
                                   tolerance=1e-4)
    assert info.converged == 1 and info.iterations < 60
    it = int(info.iterations)
    _e2e_check(oracle, P, n, d, k, it, C0, C, M, L.view(np.uint32),
               lambda: ckm.kmeans_run(P, d, k, it - 1, C0, pipeline=pipeline, spatial_order=1)[0])


def test_pipeline_double_types(ckm, oracle, cuda):
    n, d, k, iters = 20000, 3, 6, 5
    P = blobs(n, d, k, seed=98).astype(np.float64)
    C0 = oracle.first_x_f32(P.astype(np.float32), n, d, k).astype(np.float64)
    for pipeline in ("single_stage", "three_stage", "single_stage_buffered", "three_stage_buffered"):
        C, M, L, _ = ckm.kmeans_run(P, d, k, iters, C0, pipeline=pipeline,
                                    chunk_bytes=(6000 * d * 8 if "buffered" in pipeline else 0))
        Cr, Mr, Lr = oracle.lloyd_f64(P, n, d, k, iters, C0)
        assert np.array_equal(L, Lr), pipeline
        assert np.array_equal(M, Mr), pipeline
        assert np.allclose(C, Cr, rtol=1e-12, atol=1e-12), pipeline


def test_unknown_strategy_is_rejected(ckm, cuda):
    P = blobs(1000, 2, 3, seed=1)
    C0 = P.reshape(2, 1000)[:, :3].copy().reshape(-1)
    with pytest.raises(ckm.CkmError) as e:
        ckm.kmeans_run(P, 2, 3, 1, C0, pipeline="single_stage", fused_strategy="no_such_strategy")
    assert e.value.status == -8
    with pytest.raises(ckm.CkmError) as e:
        ckm.kmeans_run(P, 2, 3, 1, C0, pipeline="three_stage", mass_update_strategy="bogus")
    assert e.value.status == -8
    with pytest.raises(ckm.CkmError) as e:
        ckm.kmeans_run(P, 2, 3, 1, C0, pipeline="warp_drive")
    assert e.value.status == -8


def test_generator_is_deterministic_and_chunkable(ckm, cuda):
    import torch
    n, d = 100000, 5
    a = torch.empty(n * d, dtype=torch.float32, device=cuda)
    b = torch.empty(n * d, dtype=torch.float32, device=cuda)
    ckm.generate_mixture(a, n, d, 16, seed=42, sigma=(0.5, 2.0))
    ckm.generate_mixture(b, n, d, 16, seed=42, sigma=(0.5, 2.0))
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    # the second half generated on its own (first_point offset, row stride n)
    c = torch.zeros(n * d, dtype=torch.float32, device=cuda)
    half = n // 2
    ckm.generate_mixture(c[half:], n - half, d, 16, seed=42, sigma=(0.5, 2.0), first_point=half, stride=n)
    torch.cuda.synchronize()
    A = a.view(d, n)[:, half:]
    C = c.view(d, n)[:, half:]
    assert torch.equal(A, C)
    x = a.cpu().numpy()
    assert np.isfinite(x).all() and np.abs(x).max() < 40.0


def test_generator_ex_laws(ckm, cuda):
    """Normal centres, log-uniform sigmas, Dirichlet(1) weights: deterministic,
    chunkable, finite, and the spread follows the centre law."""
    import torch
    n, d, blobs = 200000, 8, 64
    a = torch.empty(n * d, dtype=torch.float32, device=cuda)
    b = torch.empty(n * d, dtype=torch.float32, device=cuda)
    kw = dict(center=("normal", 0.0, 2.0), sigma=("loguniform", 0.25, 1.0), dirichlet=True)
    ckm.generate_mixture_ex(a, n, d, blobs, 5, **kw)
    ckm.generate_mixture_ex(b, n, d, blobs, 5, **kw)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    c = torch.zeros(n * d, dtype=torch.float32, device=cuda)
    ckm.generate_mixture_ex(c[1000:], n - 1000, d, blobs, 5, first_point=1000, stride=n, **kw)
    torch.cuda.synchronize()
    assert torch.equal(a.view(d, n)[:, 1000:], c.view(d, n)[:, 1000:])
    x = a.cpu().numpy()
    assert np.isfinite(x).all()
    assert 1.0 < x.std() < 4.0          # N(0, 4) centres plus sigma <= 1
    assert abs(x.mean()) < 1.0


@pytest.mark.parametrize("pipeline", ["single_stage", "three_stage", "single_stage_buffered",
                                      "three_stage_buffered"])
def test_convergence_stops_early(ckm, oracle, cuda, pipeline):
    """kmeans.converge: the run stops after the first iteration whose relative
    centroid shift is below the tolerance, with the same result as a fixed run
    of that many iterations."""
    n, d, k = 60000, 3, 6
    P = blobs(n, d, k, seed=5, spread=8.0, sigma=0.6)
    C0 = oracle.first_x_f32(P, n, d, k)
    extra = {}
    if pipeline.endswith("buffered"):
        extra = dict(chunk_bytes=16000 * d * 4, device_budget_bytes=(16000 * (d + 1) * 4) * 5 + (1 << 20) + 65536)
    C, M, L, info = ckm.kmeans_run(P, d, k, 200, C0, pipeline=pipeline, converge=True, tolerance=1e-5, **extra)
    assert info.converged == 1 and 2 <= info.iterations < 200
    assert 0.0 <= info.last_shift < 1e-5
    C2, M2, L2, info2 = ckm.kmeans_run(P, d, k, info.iterations, C0, pipeline=pipeline, **extra)
    assert info2.converged == 0 and info2.iterations == info.iterations
    assert np.array_equal(L, L2) and np.array_equal(M, M2)
    assert np.allclose(C, C2, rtol=1e-6, atol=1e-6 * np.abs(P).max())
    _e2e_check(oracle, P, n, d, k, info.iterations, C0, C, M, L,
               lambda: ckm.kmeans_run(P, d, k, info.iterations - 1, C0, pipeline=pipeline, **extra)[0])


def test_centroid_shift_matches_numpy(ckm, cuda):
    """ckm_centroid_shift_*: max |new - old| / max |old|, NaN entries skipped."""
    import ctypes
    import torch
    rng = np.random.default_rng(9)
    d, k = 7, 33
    old = rng.normal(size=k * d).astype(np.float32)
    new = (old + rng.normal(scale=1e-3, size=k * d)).astype(np.float32)
    new[5] = np.nan  # an empty cluster's coordinate
    want = np.nanmax(np.abs(new.astype(np.float64) - old)) / np.abs(old).max()
    dO, dN = to_dev(old, cuda), to_dev(new, cuda)
    out = torch.zeros(1, dtype=torch.float32, device=cuda)
    L = ckm.lib()
    L.ckm_centroid_shift_f32.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    s = torch.cuda.current_stream()
    assert L.ckm_centroid_shift_f32(d, k, dO.data_ptr(), dN.data_ptr(), out.data_ptr(), s.cuda_stream) == 0
    torch.cuda.synchronize()
    assert abs(float(out.item()) - want) <= 1e-6 * want


def test_release_cached_memory_after_runs(ckm, oracle, cuda):
    """The strategies keep their device buffers in the default stream-ordered
    pool between runs; a second run of the same shape gives the same result,
    and ckm_release_cached_memory returns the cached memory."""
    n, d, k = 50000, 8, 12
    P = blobs(n, d, 6, seed=5)
    C0 = oracle.first_x_f32(P, n, d, k)
    outs = []
    for _ in range(2):
        C, M, L, _info = ckm.kmeans_run(P, d, k, 4, C0)
        outs.append((C.copy(), M.copy(), L.copy()))
    assert np.array_equal(outs[0][2], outs[1][2])
    assert np.array_equal(outs[0][1], outs[1][1])
    assert ckm.lib().ckm_release_cached_memory() == 0
