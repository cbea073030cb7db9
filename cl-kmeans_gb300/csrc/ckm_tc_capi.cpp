// C ABI of the tensor-core fused iteration (declared in include/ckm.h).
#include <cuda_runtime.h>

#include "ckm_internal.h"
#include "ckm_tc.h"

using namespace ckm;

extern "C" {

size_t ckm_tc_points_bytes(uint64_t n, uint32_t d) { return tc_layout(n, d, 1).pts_total; }

size_t ckm_tc_workspace_bytes(uint64_t n, uint32_t d, uint32_t k) { return tc_layout(n, d, k).ws_total; }

int ckm_tc_supported(uint32_t d, uint32_t k) { return tc_supported(d, k) ? 1 : 0; }

int ckm_tc_prepare_points_ex(uint32_t d, uint64_t n, const float* points, void* tc_points, size_t bytes,
                             int precision, ckm_stream_t stream) {
    if (d == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features must be >= 1");
    if (!tc_points || (n > 0 && !points)) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (precision != CKM_TC_FP16 && precision != CKM_TC_BF16)
        return fail(CKM_ERR_INVALID_ARGUMENT, "precision must be CKM_TC_FP16 or CKM_TC_BF16");
    if (bytes < ckm_tc_points_bytes(n, d)) return fail(CKM_ERR_SCRATCH_TOO_SMALL, "tc_points smaller than ckm_tc_points_bytes");
    if (reinterpret_cast<uintptr_t>(tc_points) % 256) return fail(CKM_ERR_INVALID_ARGUMENT, "tc_points must be 256-byte aligned");
    return tc_prepare_points(points, n, d, tc_points, precision, (cudaStream_t)stream);
}

int ckm_tc_prepare_points(uint32_t d, uint64_t n, const float* points, void* tc_points, size_t bytes,
                          ckm_stream_t stream) {
    return ckm_tc_prepare_points_ex(d, n, points, tc_points, bytes, CKM_TC_FP16, stream);
}

int ckm_tc_sort_points(uint32_t d, uint64_t n, uint32_t k, const void* tc_points, void* sorted_tc_points,
                       size_t bytes, const void* workspace, size_t workspace_bytes, ckm_stream_t stream) {
    if (d == 0 || k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features and num_clusters must be >= 1");
    if (!tc_points || !sorted_tc_points || !workspace) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (tc_points == sorted_tc_points) return fail(CKM_ERR_INVALID_ARGUMENT, "the sorted set needs its own buffer");
    if (bytes < ckm_tc_points_bytes(n, d)) return fail(CKM_ERR_SCRATCH_TOO_SMALL, "sorted_tc_points smaller than ckm_tc_points_bytes");
    if (workspace_bytes < ckm_tc_workspace_bytes(n, d, k))
        return fail(CKM_ERR_SCRATCH_TOO_SMALL, "workspace smaller than ckm_tc_workspace_bytes(n, d, k)");
    if (reinterpret_cast<uintptr_t>(tc_points) % 256 || reinterpret_cast<uintptr_t>(sorted_tc_points) % 256 ||
        reinterpret_cast<uintptr_t>(workspace) % 256)
        return fail(CKM_ERR_INVALID_ARGUMENT, "buffers must be 256-byte aligned");
    return tc_sort_points(n, d, k, tc_points, sorted_tc_points, workspace, (cudaStream_t)stream);
}

int ckm_tc_counters(const void* workspace, uint32_t* counters, ckm_stream_t stream) {
    if (!workspace || !counters) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    // nflagged, error, resolved, overflowed: the first four words of the workspace
    cudaError_t e = cudaMemcpyAsync(counters, workspace, 4 * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                    (cudaStream_t)stream);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "ckm_tc_counters copy");
}

int ckm_tc_fused_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, const void* tc_points,
                     const float* old_centroids, float* new_centroids, uint32_t* labels, uint32_t* masses,
                     void* scratch, size_t scratch_bytes, void* workspace, size_t workspace_bytes, int mode,
                     uint32_t* stats, ckm_stream_t stream) {
    if (d == 0 || k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features and num_clusters must be >= 1");
    if (mode != CKM_MODE_DEFER && mode != CKM_MODE_FINALIZE && mode != CKM_MODE_ACCUMULATE)
        return fail(CKM_ERR_INVALID_ARGUMENT, "bad mode");
    if (!tc_supported(d, k)) return fail(CKM_ERR_UNSUPPORTED, "tensor-core path: needs a GB300/B-series GPU and d <= 256");
    if (!scratch || scratch_bytes < scratch_layout(d, k).total)
        return fail(CKM_ERR_SCRATCH_TOO_SMALL, "scratch smaller than ckm_scratch_bytes(d, k)");
    if (reinterpret_cast<uintptr_t>(scratch) % 16) return fail(CKM_ERR_INVALID_ARGUMENT, "scratch must be 16-byte aligned");
    if (!workspace || workspace_bytes < ckm_tc_workspace_bytes(n, d, k))
        return fail(CKM_ERR_SCRATCH_TOO_SMALL, "workspace smaller than ckm_tc_workspace_bytes(n, d, k)");
    if (reinterpret_cast<uintptr_t>(workspace) % 256) return fail(CKM_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    if (!tc_points || reinterpret_cast<uintptr_t>(tc_points) % 256)
        return fail(CKM_ERR_INVALID_ARGUMENT, "tc_points NULL or not 256-byte aligned");
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!old_centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "old_centroids NULL");
    if (mode != CKM_MODE_DEFER && (!new_centroids || !masses)) return fail(CKM_ERR_INVALID_ARGUMENT, "outputs NULL");
    TcArgs a;
    a.points = points;
    a.tc_points = tc_points;
    a.centroids = old_centroids;
    a.new_centroids = new_centroids;
    a.labels = labels;
    a.masses = masses;
    a.scratch = scratch_view(scratch, scratch_layout(d, k));
    a.workspace = workspace;
    a.stats = reinterpret_cast<unsigned int*>(stats);
    a.n = n;
    a.d = d;
    a.k = k;
    a.mode = mode;
    return tc_iteration(a, (cudaStream_t)stream);
}

}  // extern "C"
