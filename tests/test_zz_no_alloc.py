"""The allocation-free fused entry point, ckm_fused_f32_noalloc.

It exists for callers that cannot allocate device memory: a plugin inside a
framework that owns all device memory, a loop that must never call
cudaMalloc/cudaFree, a caller that only has its input and output buffers.
Its FP64 merge scratch is a fixed built-in device array that all calls
share, so this test checks that two calls in a row each give the same result
as ckm_fused_f32 with caller-provided scratch (labels and masses exactly,
centroids within the fused tests' tolerance), and that sizes beyond the
built-in array are refused.  It lives in its own file, collected last.
"""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu

CENTROID_RTOL = 2e-6
CENTROID_ATOL_SCALE = 2e-6


def _run(ckm, cuda, P, n, d, k, C, noalloc, mode=1, acc_init=None):
    import torch
    dP = torch.from_numpy(P).to(cuda)
    dC = torch.from_numpy(C).to(cuda)
    if acc_init is None:
        dN = torch.zeros(k * d, dtype=torch.float32, device=cuda)
        dM = torch.zeros(k, dtype=torch.int32, device=cuda)
    else:
        dN = torch.full((k * d,), acc_init[0], dtype=torch.float32, device=cuda)
        dM = torch.full((k,), acc_init[1], dtype=torch.int32, device=cuda)
    dL = torch.zeros(n, dtype=torch.int32, device=cuda)
    if noalloc:
        ckm.fused_noalloc(dP, dC, dN, dL, dM, n, d, k, mode)
    else:
        S = ckm.new_scratch(d, k, cuda)
        ckm.fused(dP, dC, dN, dL, dM, S, n, d, k, mode)
    torch.cuda.synchronize()
    return dN.cpu().numpy(), dM.cpu().numpy(), dL.cpu().numpy()


def _same(ref, got, scale):
    Cr, Mr, Lr = ref
    Cg, Mg, Lg = got
    assert np.array_equal(Lr, Lg), "labels differ"
    assert np.array_equal(Mr, Mg), "masses differ"
    nan = np.isnan(Cr)
    assert np.array_equal(nan, np.isnan(Cg))
    err = np.abs(Cg[~nan].astype(np.float64) - Cr[~nan])
    assert np.all(err <= CENTROID_RTOL * np.abs(Cr[~nan]) + CENTROID_ATOL_SCALE * scale)


def test_noalloc_two_calls_match_scratch_entry_point(ckm, oracle, cuda):
    # first call: d = 4, k = 16 (low-d kernel); second call: a different
    # shape on the same built-in scratch, so stale contents would show up
    for (n, d, k, seed) in [(100003, 4, 16, 1), (50000, 3, 40, 2)]:
        P = blobs(n, d, k, seed=seed)
        C = oracle.first_x_f32(P, n, d, k)
        ref = _run(ckm, cuda, P, n, d, k, C, noalloc=False)
        got = _run(ckm, cuda, P, n, d, k, C, noalloc=True)
        _same(ref, got, float(np.abs(P).max()))
        # and directly against the oracle: the reference's labels and masses
        want = oracle.label_f32(P, n, d, k, C)
        assert np.array_equal(got[2].view(np.uint32), want)
        assert np.array_equal(got[1].view(np.uint32), oracle.mass_u32(want, k))


def test_noalloc_repeated_calls_and_accumulate_mode(ckm, oracle, cuda):
    n, d, k = 30000, 20, 12          # generic kernel path
    P = blobs(n, d, k, seed=3)
    C = oracle.first_x_f32(P, n, d, k)
    ref = _run(ckm, cuda, P, n, d, k, C, noalloc=False)
    for _ in range(2):
        _same(ref, _run(ckm, cuda, P, n, d, k, C, noalloc=True), float(np.abs(P).max()))
    # reference functor contract: += into sums and masses
    refA = _run(ckm, cuda, P, n, d, k, C, noalloc=False, mode=2, acc_init=(0.5, 7))
    gotA = _run(ckm, cuda, P, n, d, k, C, noalloc=True, mode=2, acc_init=(0.5, 7))
    _same(refA, gotA, float(np.abs(P).max()) * 1000)


def test_noalloc_allocates_nothing_after_setup(ckm, oracle, cuda):
    """After the first call (set-up: the array's address, the kernels'
    module), further calls leave the device's free memory and torch's
    allocator untouched: no cudaMalloc, no allocating library routine."""
    import torch
    shapes = [(60000, 4, 16, 5), (20000, 20, 12, 6)]     # low-d and generic kernels
    bufs = []
    for n, d, k, seed in shapes:
        P = blobs(n, d, k, seed=seed)
        C = oracle.first_x_f32(P, n, d, k)
        bufs.append((torch.from_numpy(P).to(cuda), torch.from_numpy(C).to(cuda),
                     torch.zeros(k * d, dtype=torch.float32, device=cuda), torch.zeros(n, dtype=torch.int32, device=cuda),
                     torch.zeros(k, dtype=torch.int32, device=cuda), n, d, k))
    for dP, dC, dN, dL, dM, n, d, k in bufs:            # set-up calls
        ckm.fused_noalloc(dP, dC, dN, dL, dM, n, d, k)
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(5):
        for dP, dC, dN, dL, dM, n, d, k in bufs:
            ckm.fused_noalloc(dP, dC, dN, dL, dM, n, d, k)
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_builtin_scratch(ckm, cuda):
    import torch
    d, k = 128, 1024                     # needs ~1 MiB of scratch
    t = torch.zeros(16, dtype=torch.float32, device=cuda)
    with pytest.raises(ckm.CkmError) as e:
        ckm.fused_noalloc(t, t, t, t, t, 4, d, k)
    assert e.value.status == -3
    assert "built-in scratch" in str(e.value)
    with pytest.raises(ckm.CkmError) as e:  # DEFER would keep sums in the shared array
        ckm.fused_noalloc(t, t, t, t, t, 4, 4, 4, mode=0)
    assert e.value.status == -1
