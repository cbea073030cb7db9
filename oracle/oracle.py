"""ctypes front-end for the oracle (oracle/ckm_oracle.c) and, when it was
built, for the reference's own KmeansNaive (oracle/_ref/libckm_ref_naive.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU legs as the checker.  The product library never uses it.

Arrays follow the reference layout: points column-major ``P[f * n + p]``
(lloyd_fused_feature_sum.cl:77-79), centroids column-major ``C[f * k + c]``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libckm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libckm_ref_naive.so")

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32

_lib = None
_ref = None


def build():
    """Compile the oracle with its Makefile (fast; portable flags)."""
    subprocess.run(["make", "-s", "-C", HERE, "libckm_oracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO) or (
            os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(HERE, "ckm_oracle.c"))
        ):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.ckm_oracle_label_f32.argtypes = [_f32p, _u64, _u32, _u32, _f32p, _u32p]
        L.ckm_oracle_label_f64.argtypes = [_f64p, _u64, _u32, _u32, _f64p, _u64p]
        L.ckm_oracle_mass_u32.argtypes = [_u32p, _u64, _u32, _u32p]
        L.ckm_oracle_update_f32.argtypes = [_f32p, _u64, _u32, _u32, _u32p, _f32p, _u32p]
        L.ckm_oracle_update_f64.argtypes = [_f64p, _u64, _u32, _u32, _u64p, _f64p, _u64p]
        L.ckm_oracle_lloyd_f32.argtypes = [_f32p, _u64, _u32, _u32, _u32, _f32p, _u32p, _u32p]
        L.ckm_oracle_lloyd_f64.argtypes = [_f64p, _u64, _u32, _u32, _u32, _f64p, _u64p, _u64p]
        L.ckm_oracle_first_x_f32.argtypes = [_f32p, _u64, _u32, _u32, _f32p]
        L.ckm_oracle_label_gap_f64.argtypes = [_f32p, _u64, _u32, _u32, _f32p, _u32p, _f64p, _f64p]
        L.ckm_oracle_lloyd_fp64_of_f32.argtypes = [_f32p, _u64, _u32, _u32, _u32, _f64p, _u64p, _u32p]
        L.ckm_oracle_sums_f64.argtypes = [_f32p, _u64, _u32, _u32, _u32p, _f64p, _u64p]
        L.ckm_oracle_partition_matrix.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                                  ctypes.c_size_t, ctypes.c_size_t]
        L.ckm_oracle_partition_matrix.restype = ctypes.c_int
        L.ckm_oracle_lloyd_f32_mt.argtypes = [_f32p, _u64, _u32, _u32, _u32, _f32p, _u32p, _u32p,
                                              ctypes.c_int]
        L.ckm_oracle_lloyd_f32_mt.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_SO)


def ref():
    """The reference's KmeansNaive built unchanged (None when not built)."""
    global _ref
    if _ref is None:
        if not ref_available():
            return None
        R = ctypes.CDLL(REF_SO)
        R.ckm_ref_naive_f32.argtypes = [_f32p, _u64, _u32, _u32, _u32, _f32p, _u32p, _u32p, ctypes.c_int]
        R.ckm_ref_naive_f64.argtypes = [_f64p, _u64, _u32, _u32, _u32, _f64p, _u64p, _u64p, ctypes.c_int]
        R.ckm_ref_naive_f32_timed.argtypes = [_f32p, _u64, _u32, _u32, _u32, _f32p, _u32p, _u32p, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_uint64)]
        _ref = R
    return _ref


def _cm(points):
    """(n, d) row-per-point array -> flat column-major copy, plus n, d."""
    points = np.asarray(points)
    n, d = points.shape
    return np.ascontiguousarray(points.T).reshape(-1), n, d


# ----------------------------------------------------------------------------
# Thin wrappers.  `P` is always the flat column-major array of length n*d.
# ----------------------------------------------------------------------------
def label_f32(P, n, d, k, C):
    out = np.empty(n, np.uint32)
    lib().ckm_oracle_label_f32(P, n, d, k, np.ascontiguousarray(C, np.float32), out)
    return out


def label_f64(P, n, d, k, C):
    out = np.empty(n, np.uint64)
    lib().ckm_oracle_label_f64(P, n, d, k, np.ascontiguousarray(C, np.float64), out)
    return out


def mass_u32(labels, k):
    m = np.zeros(k, np.uint32)
    lib().ckm_oracle_mass_u32(np.ascontiguousarray(labels, np.uint32), len(labels), k, m)
    return m


def update_f32(P, n, d, k, labels):
    C = np.empty(k * d, np.float32)
    m = np.empty(k, np.uint32)
    lib().ckm_oracle_update_f32(P, n, d, k, np.ascontiguousarray(labels, np.uint32), C, m)
    return C, m


def lloyd_f32(P, n, d, k, iterations, C0):
    C = np.array(C0, np.float32, copy=True)
    m = np.zeros(k, np.uint32)
    lab = np.zeros(n, np.uint32)
    lib().ckm_oracle_lloyd_f32(P, n, d, k, iterations, C, m, lab)
    return C, m, lab


def lloyd_f32_mt(P, n, d, k, iterations, C0, threads):
    C = np.array(C0, np.float32, copy=True)
    m = np.zeros(k, np.uint32)
    lab = np.zeros(n, np.uint32)
    rc = lib().ckm_oracle_lloyd_f32_mt(P, n, d, k, iterations, C, m, lab, threads)
    if rc != 0:
        raise MemoryError("oracle threaded Lloyd failed to allocate")
    return C, m, lab


def lloyd_f64(P, n, d, k, iterations, C0):
    C = np.array(C0, np.float64, copy=True)
    m = np.zeros(k, np.uint64)
    lab = np.zeros(n, np.uint64)
    lib().ckm_oracle_lloyd_f64(np.ascontiguousarray(P, np.float64), n, d, k, iterations, C, m, lab)
    return C, m, lab


def lloyd_fp64_of_f32(P, n, d, k, iterations, C0):
    C = np.array(C0, np.float64, copy=True)
    m = np.zeros(k, np.uint64)
    lab = np.zeros(n, np.uint32)
    lib().ckm_oracle_lloyd_fp64_of_f32(P, n, d, k, iterations, C, m, lab)
    return C, m, lab


def first_x_f32(P, n, d, k):
    C = np.empty(k * d, np.float32)
    lib().ckm_oracle_first_x_f32(P, n, d, k, C)
    return C


def label_gap_f64(P, n, d, k, C):
    lab = np.empty(n, np.uint32)
    gap = np.empty(n, np.float64)
    best = np.empty(n, np.float64)
    lib().ckm_oracle_label_gap_f64(P, n, d, k, np.ascontiguousarray(C, np.float32), lab, gap, best)
    return lab, gap, best


def sums_f64(P, n, d, k, labels):
    s = np.empty(k * d, np.float64)
    m = np.empty(k, np.uint64)
    lib().ckm_oracle_sums_f64(P, n, d, k, np.ascontiguousarray(labels, np.uint32), s, m)
    return s, m


def partition_matrix(src_bytes, num_dims, buffer_size):
    src = np.ascontiguousarray(np.frombuffer(src_bytes, np.uint8))
    nb = (len(src) + buffer_size - 1) // buffer_size
    dst = np.zeros(max(nb * buffer_size, 1), np.uint8)
    rc = lib().ckm_oracle_partition_matrix(src.ctypes.data, dst.ctypes.data, len(src), num_dims,
                                           buffer_size)
    return rc, dst


def ref_naive_f32(P, n, d, k, iterations, C0=None):
    R = ref()
    C = np.zeros(k * d, np.float32) if C0 is None else np.array(C0, np.float32, copy=True)
    m = np.zeros(k, np.uint32)
    lab = np.zeros(n, np.uint32)
    R.ckm_ref_naive_f32(P, n, d, k, iterations, C, m, lab, 1 if C0 is None else 0)
    return C, m, lab


def ref_naive_f32_timed(P, n, d, k, iterations, C0):
    """The reference's KmeansNaive32 from the given centroids; also returns the
    seconds of its iteration loop alone (no Matrix copies)."""
    R = ref()
    C = np.array(C0, np.float32, copy=True)
    m = np.zeros(k, np.uint32)
    lab = np.zeros(n, np.uint32)
    ns = ctypes.c_uint64(0)
    R.ckm_ref_naive_f32_timed(P, n, d, k, iterations, C, m, lab, 0, ctypes.byref(ns))
    return C, m, lab, ns.value / 1e9


def ref_naive_f64(P, n, d, k, iterations, C0=None):
    R = ref()
    C = np.zeros(k * d, np.float64) if C0 is None else np.array(C0, np.float64, copy=True)
    m = np.zeros(k, np.uint64)
    lab = np.zeros(n, np.uint64)
    R.ckm_ref_naive_f64(np.ascontiguousarray(P, np.float64), n, d, k, iterations, C, m, lab,
                        1 if C0 is None else 0)
    return C, m, lab
