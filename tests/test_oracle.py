"""The oracle (oracle/ckm_oracle.c) pinned against the reference.

1. Golden fixtures made by the reference's own KmeansNaive, compiled
   unchanged (tests/golden/make_golden.py): the oracle reproduces them
   bit-for-bit (labels, masses, centroids including NaN positions).
2. When the reference build is present (oracle/_ref), random cases are
   compared live as well.
3. Helper restatements: the first_x initialiser, the mass histogram,
   partition_matrix (buffer_helper.cpp:16-87) on the reference's
   buffer-cache test patterns.
"""
import glob
import os

import numpy as np
import pytest

from conftest import blobs

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return np.array_equal(a, b)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_reproduces_reference_golden(oracle, path):
    z = np.load(path)
    n, d, k, it = [int(x) for x in z["shape"]]
    if str(z["type"]) == "f32":
        C, M, L = oracle.lloyd_f32(z["points"], n, d, k, it, z["centroids0"])
    else:
        C, M, L = oracle.lloyd_f64(z["points"], n, d, k, it, z["centroids0"])
    assert same_bits(L, z["labels"])
    assert same_bits(M, z["masses"])
    assert same_bits(C, z["centroids"])


def test_golden_set_is_complete():
    names = {os.path.basename(p)[:-4] for p in GOLDEN}
    for want in ("c1_small", "ragged", "empty_clusters", "lattice_ties", "f64_small"):
        assert want in names


@pytest.mark.parametrize("n,d,k,it", [(3001, 4, 10, 7), (1000, 2, 64, 3), (257, 9, 5, 4)])
def test_oracle_matches_live_reference(oracle, n, d, k, it):
    if not oracle.ref_available():
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    P = blobs(n, d, max(2, k // 3), seed=n * d + k)
    C0 = oracle.first_x_f32(P, n, d, k)
    Cr, Mr, Lr = oracle.ref_naive_f32(P, n, d, k, it)
    Co, Mo, Lo = oracle.lloyd_f32(P, n, d, k, it, C0)
    assert same_bits(Lr, Lo) and same_bits(Mr, Mo) and same_bits(Cr, Co)


def test_first_x_and_mass(oracle):
    n, d, k = 7, 2, 10
    P = np.arange(n * d, dtype=np.float32)
    C = oracle.first_x_f32(P, n, d, k).reshape(d, k)
    for c in range(k):
        assert C[0, c] == P[c % n] and C[1, c] == P[n + c % n]
    labels = np.array([0, 3, 3, 9, 0, 3], np.uint32)
    assert list(oracle.mass_u32(labels, 10)) == [2, 0, 0, 3, 0, 0, 0, 0, 0, 1]


def test_threaded_port_labels_equal_serial(oracle):
    n, d, k = 20011, 4, 16
    P = blobs(n, d, k, seed=3)
    C0 = oracle.first_x_f32(P, n, d, k)
    C1, M1, L1 = oracle.lloyd_f32(P, n, d, k, 1, C0)
    C2, M2, L2 = oracle.lloyd_f32_mt(P, n, d, k, 1, C0, 4)
    assert np.array_equal(L1, L2) and np.array_equal(M1, M2)
    assert np.allclose(C1, C2, rtol=1e-6)


def _partition_py(src, num_dims, buffer_size):
    """Independent restatement of partition_matrix for the check."""
    size = len(src)
    dim_size = size // num_dims
    buf_dim = buffer_size // num_dims
    nb = (size + buffer_size - 1) // buffer_size
    out = bytearray(nb * buffer_size)
    for b in range(nb):
        for v in range(num_dims):
            real = dim_size - b * buf_dim if buf_dim * (b + 1) > dim_size else buf_dim
            out[b * buffer_size + v * real: b * buffer_size + v * real + real] = \
                src[v * dim_size + b * buf_dim: v * dim_size + b * buf_dim + real]
    return nb, bytes(out)


@pytest.mark.parametrize("pattern", ["ascending", "deadbeef", "canary"])
def test_partition_matrix(oracle, pattern):
    # the buffer-cache test patterns (test/buffer_cache.cpp:176-221)
    words = 3 * 4096 + 12
    if pattern == "ascending":
        a = np.arange(words, dtype=np.uint32)
    elif pattern == "deadbeef":
        a = np.full(words, 0xDEADBEEF, dtype=np.uint32)
    else:
        a = np.full(words, 0x13371337, dtype=np.uint32)
        a[::7] = np.arange(len(a[::7]), dtype=np.uint32)
    src = a.tobytes()
    for dims, buf in [(3, 3 * 1024), (4, 4 * 256), (1, 4096)]:
        if len(src) % dims:
            continue
        rc, dst = oracle.partition_matrix(src, dims, buf)
        nb, want = _partition_py(src, dims, buf)
        assert rc == nb
        assert bytes(dst[:len(want)]) == want
    rc, _ = oracle.partition_matrix(src, 5, 4096 * 5 + 1)
    assert rc == -1
