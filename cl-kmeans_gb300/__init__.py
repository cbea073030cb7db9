"""GB300-native Lloyd k-means: Python handle on libckm.so.

The library is C++/CUDA (kernels for sm_103a, the C ABI of include/ckm.h, and
the C++ strategy layer that mirrors the reference's AbstractKmeans /
strategies / factories).  This module only loads it with ctypes and adds thin
helpers that pass torch device tensors (plumbing for tests and bench.py).
There is no CPU fallback: every helper raises when the library is missing or
a call fails.

The directory name has a hyphen, so import it with
``importlib.import_module("cl-kmeans_gb300")``.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libckm.so")
BENCH_BIN = os.path.join(_HERE, "bin", "ckm_bench")

MODE_DEFER = 0
MODE_FINALIZE = 1
MODE_ACCUMULATE = 2

STATUS = {
    0: "CKM_OK", -1: "CKM_ERR_INVALID_ARGUMENT", -2: "CKM_ERR_UNSUPPORTED", -3: "CKM_ERR_SCRATCH_TOO_SMALL",
    -4: "CKM_ERR_CUDA", -5: "CKM_ERR_ALLOC", -6: "CKM_ERR_IO", -7: "CKM_ERR_TIMEOUT",
    -8: "CKM_ERR_UNKNOWN_STRATEGY", -9: "CKM_ERR_CANCELLED", -10: "CKM_ERR_BUDGET",
}

# Every symbol include/ckm.h declares (checked by the tests).
EXPORTS = [
    "ckm_status_string", "ckm_last_error", "ckm_version", "ckm_device_count", "ckm_launch_count",
    "ckm_release_cached_memory",
    "ckm_scratch_bytes", "ckm_scratch_init",
    "ckm_fused_f32", "ckm_fused_f64", "ckm_fused_f32_noalloc", "ckm_labeling_f32", "ckm_labeling_f64",
    "ckm_mass_update_u32", "ckm_mass_update_u64", "ckm_centroid_update_f32", "ckm_centroid_update_f64",
    "ckm_matrix_divide_row_f32", "ckm_matrix_divide_row_f64", "ckm_matrix_add_f32", "ckm_matrix_add_f64",
    "ckm_matrix_add_u32", "ckm_matrix_add_u64", "ckm_reduce_vector_parcol_u32",
    "ckm_finalize_f32", "ckm_finalize_f64", "ckm_generate_mixture_f32",
    "ckm_kmeans_run_f32", "ckm_kmeans_run_f64",
    "ckm_spatial_sort_workspace_bytes", "ckm_spatial_sort_f32", "ckm_fused_sorted_f32", "ckm_unpermute_u32",
    "ckm_labeling_sorted_f32",
]


class CkmError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        msg = "%s failed: %s" % (where, STATUS.get(status, status))
        if detail:
            msg += " (%s)" % detail
        super().__init__(msg)


class RunConfig(ctypes.Structure):
    """struct ckm_run_config (include/ckm.h)."""
    _fields_ = [
        ("pipeline", ctypes.c_char_p),
        ("fused_strategy", ctypes.c_char_p),
        ("labeling_strategy", ctypes.c_char_p),
        ("mass_update_strategy", ctypes.c_char_p),
        ("centroid_update_strategy", ctypes.c_char_p),
        ("device", ctypes.c_int),
        ("device_budget_bytes", ctypes.c_uint64),
        ("chunk_bytes", ctypes.c_uint64),
        ("converge", ctypes.c_int),
        ("tolerance", ctypes.c_double),
        ("spatial_order", ctypes.c_int),
    ]


class RunInfo(ctypes.Structure):
    """struct ckm_run_info (include/ckm.h)."""
    _fields_ = [
        ("total_time_ns", ctypes.c_uint64),
        ("h2d_bytes", ctypes.c_uint64),
        ("d2h_bytes", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
        ("iterations", ctypes.c_uint32),
        ("converged", ctypes.c_uint32),
        ("last_shift", ctypes.c_float),
    ]


_lib = None


def build(force=False, verbose=False):
    """Compile libckm.so (and ckm_bench) in-tree for sm_103a."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_ckm_build", os.path.join(_HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force, verbose=verbose)


def lib():
    """The loaded libckm.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libckm.so not built: run __graft_entry__.build() or cl-kmeans_gb300/build.py")
    L = ctypes.CDLL(LIB_PATH)
    vp, u32, u64, i32, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_size_t
    sigs = {
        "ckm_status_string": ([i32], ctypes.c_char_p),
        "ckm_last_error": ([], ctypes.c_char_p),
        "ckm_version": ([], i32),
        "ckm_device_count": ([ctypes.POINTER(ctypes.c_int)], i32),
        "ckm_launch_count": ([], u64),
        "ckm_release_cached_memory": ([], i32),
        "ckm_scratch_bytes": ([u32, u32], sz),
        "ckm_scratch_init": ([vp, sz, vp], i32),
        "ckm_fused_f32": ([u32, u64, u32, vp, vp, vp, vp, vp, vp, sz, i32, vp], i32),
        "ckm_fused_f64": ([u32, u64, u32, vp, vp, vp, vp, vp, vp, sz, i32, vp], i32),
        "ckm_fused_f32_noalloc": ([u32, u64, u32, vp, vp, vp, vp, vp, i32, vp], i32),
        "ckm_labeling_f32": ([u32, u64, u32, vp, vp, vp, vp], i32),
        "ckm_labeling_f64": ([u32, u64, u32, vp, vp, vp, vp], i32),
        "ckm_mass_update_u32": ([u64, u32, vp, vp, vp], i32),
        "ckm_mass_update_u64": ([u64, u32, vp, vp, vp], i32),
        "ckm_centroid_update_f32": ([u32, u64, u32, vp, vp, vp, vp, vp, sz, i32, vp], i32),
        "ckm_centroid_update_f64": ([u32, u64, u32, vp, vp, vp, vp, vp, sz, i32, vp], i32),
        "ckm_matrix_divide_row_f32": ([u32, u32, vp, vp, vp], i32),
        "ckm_matrix_divide_row_f64": ([u32, u32, vp, vp, vp], i32),
        "ckm_matrix_add_f32": ([u64, vp, vp, vp], i32),
        "ckm_matrix_add_f64": ([u64, vp, vp, vp], i32),
        "ckm_matrix_add_u32": ([u64, vp, vp, vp], i32),
        "ckm_matrix_add_u64": ([u64, vp, vp, vp], i32),
        "ckm_reduce_vector_parcol_u32": ([u64, u64, vp, vp], i32),
        "ckm_finalize_f32": ([u32, u32, vp, vp, vp, sz, vp], i32),
        "ckm_finalize_f64": ([u32, u32, vp, vp, vp, sz, vp], i32),
        "ckm_generate_mixture_f32": ([u32, u64, u32, u64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_float, u64, vp, u64, vp], i32),
        "ckm_kmeans_run_f32": ([ctypes.POINTER(RunConfig), u32, u32, u64, u32, vp, vp, vp, vp,
                                ctypes.POINTER(RunInfo)], i32),
        "ckm_kmeans_run_f64": ([ctypes.POINTER(RunConfig), u32, u32, u64, u32, vp, vp, vp, vp,
                                ctypes.POINTER(RunInfo)], i32),
        "ckm_spatial_sort_workspace_bytes": ([u64, u32], sz),
        "ckm_spatial_sort_f32": ([u32, u64, vp, vp, vp, vp, sz, vp], i32),
        "ckm_fused_sorted_f32": ([u32, u64, u32, vp, vp, vp, vp, vp, vp, sz, i32, vp], i32),
        "ckm_unpermute_u32": ([u64, vp, vp, vp, vp], i32),
        "ckm_labeling_sorted_f32": ([u32, u64, u32, vp, vp, vp, vp], i32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return _lib


def check(status, where):
    if status != 0:
        detail = lib().ckm_last_error()
        raise CkmError(status, where, detail.decode() if detail else "")
    return status


# ----------------------------------------------------------------------------
# torch plumbing (device memory and streams only)
# ----------------------------------------------------------------------------
def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def scratch_bytes(d, k):
    return int(lib().ckm_scratch_bytes(d, k))


def new_scratch(d, k, device="cuda"):
    """Zeroed FP64 merge scratch for (d, k) as a torch uint8 tensor."""
    import torch
    t = torch.empty(scratch_bytes(d, k), dtype=torch.uint8, device=device)
    check(lib().ckm_scratch_init(_p(t), t.numel(), _stream()), "ckm_scratch_init")
    return t


def _is64(t):
    import torch
    return t.dtype == torch.float64


def fused(points, old_centroids, new_centroids, labels, masses, scratch, n, d, k, mode=MODE_FINALIZE,
          stream=None):
    """ckm_fused_{f32,f64}: label + mass + sums (+ divide) in one launch."""
    fn = lib().ckm_fused_f64 if _is64(points) else lib().ckm_fused_f32
    check(fn(d, n, k, _p(points), _p(old_centroids), _p(new_centroids), _p(labels), _p(masses), _p(scratch),
             scratch.numel(), mode, _stream(stream)), "ckm_fused")


def spatial_sort(points, n, d, stream=None, with_perm=True):
    """ckm_spatial_sort_f32: (sorted column-major points, perm) on the points'
    device; perm[q] is the index in `points` of sorted point q (None when
    with_perm is False: the sort then moves no indices)."""
    import torch
    L = lib()
    out = torch.empty_like(points)
    perm = torch.empty(n, dtype=torch.int32, device=points.device) if with_perm else None
    ws = torch.empty(int(L.ckm_spatial_sort_workspace_bytes(n, d)), dtype=torch.uint8, device=points.device)
    check(L.ckm_spatial_sort_f32(d, n, _p(points), _p(out), _p(perm) if with_perm else None, _p(ws), ws.numel(),
                                 _stream(stream)), "ckm_spatial_sort_f32")
    return out, perm


def fused_sorted(points, old_centroids, new_centroids, labels, masses, scratch, n, d, k, mode=MODE_FINALIZE,
                 stream=None):
    """ckm_fused_sorted_f32: ckm_fused_f32 with per-warp box pruning (for
    spatially ordered points); labels in the order of `points`."""
    check(lib().ckm_fused_sorted_f32(d, n, k, _p(points), _p(old_centroids), _p(new_centroids), _p(labels),
                                     _p(masses), _p(scratch), scratch.numel(), mode, _stream(stream)),
          "ckm_fused_sorted_f32")


def unpermute(perm, labels_in, labels_out, n, stream=None):
    """ckm_unpermute_u32: labels_out[perm[q]] = labels_in[q]."""
    check(lib().ckm_unpermute_u32(n, _p(perm), _p(labels_in), _p(labels_out), _stream(stream)), "ckm_unpermute_u32")


def fused_noalloc(points, old_centroids, new_centroids, labels, masses, n, d, k, mode=MODE_FINALIZE,
                  stream=None):
    """ckm_fused_f32_noalloc: the fused iteration with the library's built-in
    scratch, for callers that cannot allocate (no scratch argument)."""
    check(lib().ckm_fused_f32_noalloc(d, n, k, _p(points), _p(old_centroids), _p(new_centroids), _p(labels),
                                      _p(masses), mode, _stream(stream)), "ckm_fused_f32_noalloc")


def labeling(points, centroids, labels, n, d, k, stream=None):
    fn = lib().ckm_labeling_f64 if _is64(points) else lib().ckm_labeling_f32
    check(fn(d, n, k, _p(points), _p(centroids), _p(labels), _stream(stream)), "ckm_labeling")


def mass_update(labels, masses, n, k, stream=None):
    import torch
    fn = lib().ckm_mass_update_u64 if labels.dtype in (torch.int64, torch.uint64) else lib().ckm_mass_update_u32
    check(fn(n, k, _p(labels), _p(masses), _stream(stream)), "ckm_mass_update")


def centroid_update(points, centroids, labels, masses, scratch, n, d, k, mode=MODE_ACCUMULATE, stream=None):
    fn = lib().ckm_centroid_update_f64 if _is64(points) else lib().ckm_centroid_update_f32
    check(fn(d, n, k, _p(points), _p(centroids), _p(labels), _p(masses), _p(scratch), scratch.numel(), mode,
             _stream(stream)), "ckm_centroid_update")


def finalize(centroids, masses, scratch, d, k, stream=None):
    fn = lib().ckm_finalize_f64 if _is64(centroids) else lib().ckm_finalize_f32
    check(fn(d, k, _p(centroids), _p(masses), _p(scratch), scratch.numel(), _stream(stream)), "ckm_finalize")


def divide_row(matrix, masses, d, k, stream=None):
    fn = lib().ckm_matrix_divide_row_f64 if _is64(matrix) else lib().ckm_matrix_divide_row_f32
    check(fn(d, k, _p(matrix), _p(masses), _stream(stream)), "ckm_matrix_divide_row")


def reduce_vector_parcol(data, num_cols, num_rows, stream=None):
    check(lib().ckm_reduce_vector_parcol_u32(num_cols, num_rows, _p(data), _stream(stream)),
          "ckm_reduce_vector_parcol_u32")


def generate_mixture(points, n, d, blobs, seed, center=(-10.0, 10.0), sigma=(1.0, 1.0), first_point=0,
                     stride=None, stream=None):
    """Fills a column-major float32 device tensor with the seeded mixture."""
    check(lib().ckm_generate_mixture_f32(d, n, blobs, seed, center[0], center[1], sigma[0], sigma[1], first_point,
                                         _p(points), n if stride is None else stride, _stream(stream)),
          "ckm_generate_mixture_f32")


def launch_count():
    return int(lib().ckm_launch_count())


def kmeans_run(points, d, k, iterations, centroids, pipeline="single_stage", fused_strategy="feature_sum",
               labeling_strategy="unroll_vector", mass_update_strategy="part_local",
               centroid_update_strategy="feature_sum", device=0, device_budget_bytes=0, chunk_bytes=0,
               masses=None, labels=None, converge=False, tolerance=0.0, spatial_order=0):
    """AbstractKmeans::operator() over HOST numpy arrays (column-major flat
    points and centroids).  converge: stop once the relative centroid shift
    falls below tolerance (default 1e-4).  Returns (centroids, masses,
    labels, RunInfo)."""
    import numpy as np
    f64 = points.dtype == np.float64
    P = np.ascontiguousarray(points, np.float64 if f64 else np.float32)
    n = P.size // d
    C = np.array(centroids, np.float64 if f64 else np.float32, copy=True)
    it = np.uint64 if f64 else np.uint32
    M = np.zeros(k, it) if masses is None else masses
    Lb = np.zeros(n, it) if labels is None else labels
    cfg = RunConfig(pipeline.encode(), fused_strategy.encode(), labeling_strategy.encode(),
                    mass_update_strategy.encode(), centroid_update_strategy.encode(), device,
                    device_budget_bytes, chunk_bytes, 1 if converge else 0, float(tolerance), int(spatial_order))
    info = RunInfo()
    fn = lib().ckm_kmeans_run_f64 if f64 else lib().ckm_kmeans_run_f32
    check(fn(ctypes.byref(cfg), iterations, d, n, k, P.ctypes.data, C.ctypes.data, M.ctypes.data,
             Lb.ctypes.data, ctypes.byref(info)), "ckm_kmeans_run")
    return C, M, Lb, info


# ----------------------------------------------------------------------------
# Batched jobs (ckm_batch_*)
# ----------------------------------------------------------------------------
class BatchJob(ctypes.Structure):
    """struct ckm_batch_job (include/ckm.h)."""
    _fields_ = [
        ("points", ctypes.c_void_p),
        ("centroids", ctypes.c_void_p),
        ("labels", ctypes.c_void_p),
        ("masses", ctypes.c_void_p),
        ("num_points", ctypes.c_uint64),
        ("num_features", ctypes.c_uint32),
        ("num_clusters", ctypes.c_uint32),
    ]


class BatchOptions(ctypes.Structure):
    """struct ckm_batch_options (include/ckm.h)."""
    _fields_ = [
        ("tile_points", ctypes.c_uint32),
        ("ctas_per_sm", ctypes.c_uint32),
        ("flush_tiles", ctypes.c_uint32),
        ("autotune", ctypes.c_int),
        ("tolerance", ctypes.c_float),
        ("max_iterations", ctypes.c_uint32),
    ]


_BATCH_SIGS = {
    "ckm_batch_create": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                          ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_step": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_run": ([ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_sync": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_status": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_set_active": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_batch_info": ([ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_uint32)] * 4, ctypes.c_int),
    "ckm_batch_destroy": ([ctypes.c_void_p], ctypes.c_int),
}
EXPORTS += list(_BATCH_SIGS)


def _batch_lib():
    L = lib()
    if not getattr(L, "_batch_sigs", False):
        for name, (args, res) in _BATCH_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        L._batch_sigs = True
    return L


class Batch:
    """Owns a ckm_batch handle over torch device tensors (per job: points,
    centroids, labels, masses).  The tensors must outlive the batch."""

    def __init__(self, jobs, tile_points=0, ctas_per_sm=0, flush_tiles=0, autotune=False, stream=None,
                 tolerance=0.0, max_iterations=0):
        L = _batch_lib()
        self._keep = jobs
        arr = (BatchJob * len(jobs))()
        for i, j in enumerate(jobs):
            arr[i] = BatchJob(j["points"].data_ptr(), j["centroids"].data_ptr(), j["labels"].data_ptr(),
                              j["masses"].data_ptr(), j["n"], j["d"], j["k"])
        opt = BatchOptions(tile_points, ctas_per_sm, flush_tiles, 1 if autotune else 0, tolerance, max_iterations)
        h = ctypes.c_void_p()
        check(L.ckm_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(jobs), ctypes.byref(opt), ctypes.byref(h),
                                 _stream(stream)), "ckm_batch_create")
        self.h = h
        self.n_jobs = len(jobs)

    def step(self, stream=None):
        check(_batch_lib().ckm_batch_step(self.h, _stream(stream)), "ckm_batch_step")

    def run(self, iterations, use_graph=True, stream=None):
        check(_batch_lib().ckm_batch_run(self.h, iterations, 1 if use_graph else 0, _stream(stream)), "ckm_batch_run")

    def sync(self, stream=None):
        check(_batch_lib().ckm_batch_sync(self.h, _stream(stream)), "ckm_batch_sync")

    def status(self, stream=None):
        import numpy as np
        sh = np.zeros(self.n_jobs, np.float32)
        it = np.zeros(self.n_jobs, np.uint32)
        check(_batch_lib().ckm_batch_status(self.h, sh.ctypes.data, it.ctypes.data, _stream(stream)),
              "ckm_batch_status")
        return sh, it

    def set_active(self, active, stream=None):
        import numpy as np
        a = np.ascontiguousarray(np.asarray(active, np.uint8))
        check(_batch_lib().ckm_batch_set_active(self.h, a.ctypes.data, _stream(stream)), "ckm_batch_set_active")

    def info(self):
        v = [ctypes.c_uint32() for _ in range(4)]
        check(_batch_lib().ckm_batch_info(self.h, *[ctypes.byref(x) for x in v]), "ckm_batch_info")
        return dict(zip(("grid", "tile_points", "ctas_per_sm", "segments"), (x.value for x in v)))

    def close(self):
        if self.h:
            _batch_lib().ckm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------
# Tensor-core fused iteration (ckm_tc_*)
# ----------------------------------------------------------------------------
_TC_SIGS = {
    "ckm_tc_points_bytes": ([ctypes.c_uint64, ctypes.c_uint32], ctypes.c_size_t),
    "ckm_tc_workspace_bytes": ([ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32], ctypes.c_size_t),
    "ckm_tc_supported": ([ctypes.c_uint32, ctypes.c_uint32], ctypes.c_int),
    "ckm_tc_prepare_points": ([ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                               ctypes.c_void_p], ctypes.c_int),
    "ckm_tc_prepare_points_ex": ([ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p], ctypes.c_int),
    "ckm_tc_counters": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_tc_sort_points": ([ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p], ctypes.c_int),
    "ckm_tc_fused_f32": ([ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32] + [ctypes.c_void_p] * 7 +
                         [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                          ctypes.c_void_p], ctypes.c_int),
}
EXPORTS += list(_TC_SIGS)


def _tc_lib():
    L = lib()
    if not getattr(L, "_tc_sigs", False):
        for name, (args, res) in _TC_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        L._tc_sigs = True
    return L


class TensorCorePoints:
    """A point set prepared for the tensor-core path (scaled fp16 rows, FP32
    rows, norm bounds, point indices) and the per-(n, d, k) workspace; torch
    device memory."""

    def __init__(self, points, n, d, stream=None, precision="fp16"):
        import torch
        L = _tc_lib()
        self.n, self.d = n, d
        nbytes = int(L.ckm_tc_points_bytes(n, d))
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=points.device)
        prec = {"fp16": 0, "bf16": 1}[precision]
        check(L.ckm_tc_prepare_points_ex(d, n, _p(points), _p(self.buf), nbytes, prec, _stream(stream)),
              "ckm_tc_prepare_points_ex")
        self.ws = {}

    def sort(self, k, stream=None):
        """ckm_tc_sort_points: reorder the set by the clusters of the last
        tc_fused call with k clusters (labels keep the caller's order)."""
        import torch
        L = _tc_lib()
        ws = self.workspace(k)
        out = torch.empty_like(self.buf)
        check(L.ckm_tc_sort_points(self.d, self.n, k, _p(self.buf), _p(out), out.numel(), _p(ws), ws.numel(),
                                   _stream(stream)), "ckm_tc_sort_points")
        self.buf = out

    def counters(self, k, out, stream=None):
        """ckm_tc_counters into the int32 device tensor out[4]: rechecked,
        error, resolved among 2+ candidates, overflowed."""
        check(_tc_lib().ckm_tc_counters(_p(self.workspace(k)), _p(out), _stream(stream)), "ckm_tc_counters")

    def workspace(self, k):
        import torch
        if k not in self.ws:
            b = int(_tc_lib().ckm_tc_workspace_bytes(self.n, self.d, k))
            self.ws[k] = torch.empty(b, dtype=torch.uint8, device=self.buf.device)
        return self.ws[k]


def tc_supported(d, k):
    return bool(_tc_lib().ckm_tc_supported(d, k))


def tc_fused(points, tcp, old_centroids, new_centroids, labels, masses, scratch, n, d, k, mode=MODE_FINALIZE,
             stats=None, stream=None):
    """ckm_tc_fused_f32: one Lloyd iteration with tensor-core distances,
    certified labels and exact recheck of near-ties."""
    ws = tcp.workspace(k)
    check(_tc_lib().ckm_tc_fused_f32(d, n, k, _p(points), _p(tcp.buf), _p(old_centroids), _p(new_centroids),
                                     _p(labels), _p(masses), _p(scratch), scratch.numel(), _p(ws), ws.numel(), mode,
                                     _p(stats), _stream(stream)), "ckm_tc_fused_f32")


class MixtureSpec(ctypes.Structure):
    """struct ckm_mixture_spec (include/ckm.h)."""
    _fields_ = [
        ("num_features", ctypes.c_uint32), ("num_blobs", ctypes.c_uint32), ("seed", ctypes.c_uint64),
        ("center_dist", ctypes.c_int), ("center_a", ctypes.c_float), ("center_b", ctypes.c_float),
        ("sigma_dist", ctypes.c_int), ("sigma_lo", ctypes.c_float), ("sigma_hi", ctypes.c_float),
        ("dirichlet", ctypes.c_int),
    ]


EXPORTS.append("ckm_generate_mixture_ex_f32")
EXPORTS += ["ckm_centroid_shift_f32", "ckm_centroid_shift_f64", "ckm_transfer_probe"]


def transfer_probe(chunk_bytes, repeat=10, pinned=True, to_device=True, trials=3, device=0):
    """ckm_transfer_probe: (best, mean) GB/s of `repeat` back-to-back copies
    of chunk_bytes between host memory and the device."""
    L = lib()
    fn = L.ckm_transfer_probe
    fn.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    fn.restype = ctypes.c_int
    best, mean = ctypes.c_double(), ctypes.c_double()
    check(fn(device, chunk_bytes, repeat, 1 if pinned else 0, 1 if to_device else 0, trials, ctypes.byref(best),
             ctypes.byref(mean)), "ckm_transfer_probe")
    return best.value, mean.value


def generate_mixture_ex(points, n, d, blobs, seed, center=("uniform", -10.0, 10.0), sigma=("uniform", 1.0, 1.0),
                        dirichlet=False, first_point=0, stride=None, stream=None):
    """ckm_generate_mixture_ex_f32: centre law 'uniform' (a, b) or 'normal'
    (mean, std); sigma law 'uniform' or 'loguniform' (lo, hi); equal or
    Dirichlet(1) weights."""
    L = lib()
    fn = L.ckm_generate_mixture_ex_f32
    fn.argtypes = [ctypes.POINTER(MixtureSpec), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                   ctypes.c_void_p]
    fn.restype = ctypes.c_int
    spec = MixtureSpec(d, blobs, seed, 1 if center[0] == "normal" else 0, center[1], center[2],
                       1 if sigma[0] == "loguniform" else 0, sigma[1], sigma[2], 1 if dirichlet else 0)
    check(fn(ctypes.byref(spec), n, first_point, _p(points), n if stride is None else stride, _stream(stream)),
          "ckm_generate_mixture_ex_f32")


# ----------------------------------------------------------------------------
# Serving (ckm_server_*)
# ----------------------------------------------------------------------------
class ServerOptions(ctypes.Structure):
    """struct ckm_server_options (include/ckm.h)."""
    _fields_ = [("device", ctypes.c_int), ("device_budget_bytes", ctypes.c_uint64), ("tolerance", ctypes.c_float),
                ("max_iterations", ctypes.c_uint32), ("round_iterations", ctypes.c_uint32),
                ("large_work", ctypes.c_uint64)]


class ServerJob(ctypes.Structure):
    """struct ckm_server_job (include/ckm.h)."""
    _fields_ = [("points", ctypes.c_void_p), ("init_centroids", ctypes.c_void_p), ("centroids", ctypes.c_void_p),
                ("masses", ctypes.c_void_p), ("labels", ctypes.c_void_p), ("num_points", ctypes.c_uint64),
                ("num_features", ctypes.c_uint32), ("num_clusters", ctypes.c_uint32), ("tag", ctypes.c_uint64)]


class ServerResult(ctypes.Structure):
    """struct ckm_server_result (include/ckm.h)."""
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int), ("iterations", ctypes.c_uint32),
                ("converged", ctypes.c_uint32), ("shift", ctypes.c_float), ("lane", ctypes.c_uint32),
                ("first_round", ctypes.c_uint64), ("last_round", ctypes.c_uint64),
                ("latency_ns", ctypes.c_uint64), ("error", ctypes.c_char * 128)]


_SERVER_SIGS = {
    "ckm_server_create": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_server_submit": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_server_poll": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p], ctypes.c_int),
    "ckm_server_drain": ([ctypes.c_void_p], ctypes.c_int),
    "ckm_server_stats_get": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "ckm_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
}
EXPORTS += list(_SERVER_SIGS)


def _server_lib():
    L = lib()
    if not getattr(L, "_server_sigs", False):
        for name, (args, res) in _SERVER_SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        L._server_sigs = True
    return L


class Server:
    """ckm_server_*: a serving loop over host arrays.  submit() takes flat
    column-major float32 numpy arrays (points n*d, initial centroids k*d) and
    keeps them, and the result arrays it allocates, alive until the job's
    result is polled."""

    def __init__(self, device=0, device_budget_bytes=0, tolerance=0.0, max_iterations=0, round_iterations=0,
                 large_work=0):
        import numpy as np
        self._np = np
        L = _server_lib()
        opt = ServerOptions(device, device_budget_bytes, tolerance, max_iterations, round_iterations, large_work)
        h = ctypes.c_void_p()
        check(L.ckm_server_create(ctypes.byref(opt), ctypes.byref(h)), "ckm_server_create")
        self.h = h
        self._live = {}

    def submit(self, points, init, n, d, k, tag, labels=True, out=None):
        np = self._np
        if out is None:
            out = (np.empty(k * d, np.float32), np.empty(k, np.uint32), np.empty(n, np.uint32) if labels else None)
        C, M, Lb = out
        job = ServerJob(points.ctypes.data, init.ctypes.data, C.ctypes.data, M.ctypes.data,
                        Lb.ctypes.data if Lb is not None else None, n, d, k, tag)
        self._live[tag] = (points, init, C, M, Lb)
        rc = _server_lib().ckm_server_submit(self.h, ctypes.byref(job))
        if rc != 0:
            del self._live[tag]
        check(rc, "ckm_server_submit")

    def poll(self, max_results=4096):
        arr = (ServerResult * max_results)()
        cnt = ctypes.c_uint32()
        check(_server_lib().ckm_server_poll(self.h, ctypes.cast(arr, ctypes.c_void_p), max_results,
                                            ctypes.byref(cnt)), "ckm_server_poll")
        out = []
        for i in range(cnt.value):
            r = arr[i]
            _, _, C, M, Lb = self._live.pop(r.tag)
            out.append(dict(tag=r.tag, status=r.status, iterations=r.iterations, converged=r.converged,
                            shift=r.shift, lane=r.lane, first_round=r.first_round, last_round=r.last_round,
                            latency_ns=r.latency_ns, error=r.error.decode(errors="replace"),
                            centroids=C, masses=M, labels=Lb))
        return out

    def drain(self):
        check(_server_lib().ckm_server_drain(self.h), "ckm_server_drain")

    def stats(self):
        names = ["rounds", "job_rounds", "busy_ns", "steps_gpu_ns", "admit_ns", "retire_ns", "jobs_admitted",
                 "jobs_completed"]
        arr = (ctypes.c_uint64 * len(names))()
        check(_server_lib().ckm_server_stats_get(self.h, ctypes.cast(arr, ctypes.c_void_p)), "ckm_server_stats_get")
        return dict(zip(names, list(arr)))

    def close(self):
        if self.h:
            _server_lib().ckm_server_destroy(self.h)
            self.h = None
