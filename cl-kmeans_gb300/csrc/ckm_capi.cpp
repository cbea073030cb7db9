// extern "C" entry points of libckm.so (declared in include/ckm.h).
//
// Each entry validates its arguments (the reference asserts sizes,
// fused_feature_sum.hpp:210-220; here a bad call returns
// CKM_ERR_INVALID_ARGUMENT instead), picks the kernel for the shape and
// launches it on the caller's stream.  No entry point allocates memory.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "ckm_internal.h"

namespace ckm {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t err, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorName(err) + ": " + cudaGetErrorString(err);
    return CKM_ERR_CUDA;
}

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

ScratchLayout scratch_layout(uint32_t d, uint32_t k) {
    ScratchLayout L;
    L.sums_off = 0;
    L.mass_off = align256((size_t)d * k * sizeof(double));
    L.ctrl_off = L.mass_off + align256((size_t)k * sizeof(unsigned long long));
    L.total = L.ctrl_off + 256;
    L.ext_off = 0;
    if ((d == 32 || d == 64) && k >= 16 && k <= 256) {
        L.ext_off = L.total;
        L.total += FUSED_UMMA_EXT;
    }
    return L;
}

const DeviceInfo& device_info() {
    static std::mutex mu;
    static DeviceInfo infos[64];
    static bool have[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> g(mu);
    if (!have[dev]) {
        cudaDeviceProp p;
        std::memset(&p, 0, sizeof(p));
        if (cudaGetDeviceProperties(&p, dev) == cudaSuccess) {
            infos[dev].sm_count = p.multiProcessorCount;
            infos[dev].smem_optin = p.sharedMemPerBlockOptin;
            infos[dev].smem_per_sm = p.sharedMemPerMultiprocessor;
            infos[dev].smem_reserved = p.reservedSharedMemPerBlock;
            infos[dev].cc_major = p.major;
            infos[dev].cc_minor = p.minor;
        } else {
            infos[dev].sm_count = 1;
            infos[dev].smem_optin = 48 * 1024;
            infos[dev].smem_per_sm = 48 * 1024;
            infos[dev].smem_reserved = 0;
            infos[dev].cc_major = infos[dev].cc_minor = 0;
        }
        have[dev] = true;
    }
    return infos[dev];
}

}  // namespace ckm

using namespace ckm;

namespace {

bool valid_mode(int mode) {
    return mode == CKM_MODE_DEFER || mode == CKM_MODE_FINALIZE || mode == CKM_MODE_ACCUMULATE;
}

int check_scratch(void* scratch, size_t bytes, uint32_t d, uint32_t k) {
    if (scratch == nullptr) return fail(CKM_ERR_INVALID_ARGUMENT, "scratch is NULL");
    if (reinterpret_cast<uintptr_t>(scratch) % 16 != 0)
        return fail(CKM_ERR_INVALID_ARGUMENT, "scratch must be 16-byte aligned");
    if (bytes < scratch_layout(d, k).total)
        return fail(CKM_ERR_SCRATCH_TOO_SMALL, "scratch smaller than ckm_scratch_bytes(d, k)");
    return CKM_OK;
}

int check_shape(uint32_t d, uint64_t n, uint32_t k) {
    if (d == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features must be >= 1");
    if (k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters must be >= 1");
    if ((uint64_t)k * d > (1ull << 31)) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters * num_features too large");
    (void)n;
    return CKM_OK;
}

}  // namespace

extern "C" {

const char* ckm_status_string(int status) {
    switch (status) {
        case CKM_OK: return "ok";
        case CKM_ERR_INVALID_ARGUMENT: return "invalid argument";
        case CKM_ERR_UNSUPPORTED: return "unsupported";
        case CKM_ERR_SCRATCH_TOO_SMALL: return "scratch too small";
        case CKM_ERR_CUDA: return "CUDA error";
        case CKM_ERR_ALLOC: return "allocation failed";
        case CKM_ERR_IO: return "I/O error";
        case CKM_ERR_TIMEOUT: return "device wait timed out";
        case CKM_ERR_UNKNOWN_STRATEGY: return "unknown strategy";
        case CKM_ERR_CANCELLED: return "cancelled";
        case CKM_ERR_BUDGET: return "device memory budget exceeded";
        default: return "unknown status";
    }
}

const char* ckm_last_error(void) { return g_last_error.c_str(); }

int ckm_version(void) { return 10000; }

int ckm_device_count(int* count) {
    if (!count) return fail(CKM_ERR_INVALID_ARGUMENT, "count is NULL");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        *count = 0;
        return cuda_fail(e, "cudaGetDeviceCount");
    }
    return CKM_OK;
}

uint64_t ckm_launch_count(void) { return launch_count(); }

int ckm_release_cached_memory(void) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    cudaMemPool_t pool = nullptr;
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, 0);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "ckm_release_cached_memory");
}

size_t ckm_scratch_bytes(uint32_t num_features, uint32_t num_clusters) {
    return scratch_layout(num_features, num_clusters).total;
}

int ckm_scratch_init(void* scratch, size_t scratch_bytes, ckm_stream_t stream) {
    if (scratch == nullptr) return fail(CKM_ERR_INVALID_ARGUMENT, "scratch is NULL");
    cudaError_t e = cudaMemsetAsync(scratch, 0, scratch_bytes, (cudaStream_t)stream);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "cudaMemsetAsync(scratch)");
}

int ckm_fused_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, const float* old_centroids,
                  float* new_centroids, uint32_t* labels, uint32_t* masses, void* scratch, size_t scratch_bytes,
                  int mode, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (!valid_mode(mode)) return fail(CKM_ERR_INVALID_ARGUMENT, "mode must be DEFER, FINALIZE or ACCUMULATE");
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!old_centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "old_centroids NULL");
    if (mode != CKM_MODE_DEFER && (!new_centroids || !masses))
        return fail(CKM_ERR_INVALID_ARGUMENT, "new_centroids/masses NULL");
    FusedF32 a{points, old_centroids, labels, new_centroids, masses,
               scratch_view(scratch, scratch_layout(d, k)), n, d, k, mode};
    cudaStream_t s = (cudaStream_t)stream;
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::Fused, s);
    // d = 32 / 64 with enough points: the tensor cores (tcgen05)
    st = launch_fused_umma(a, s);
    if (st != -1000) return st;
    return launch_generic_f32(a, Pass::Fused, s);
}

int ckm_fused_sorted_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, const float* old_centroids,
                         float* new_centroids, uint32_t* labels, uint32_t* masses, void* scratch,
                         size_t scratch_bytes, int mode, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (!valid_mode(mode)) return fail(CKM_ERR_INVALID_ARGUMENT, "mode must be DEFER, FINALIZE or ACCUMULATE");
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    // labels NULL: not written (the low-d kernel only; nothing reads them)
    if (n > 0 && (!points || (!labels && !lowd_supported(d, k))))
        return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!old_centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "old_centroids NULL");
    if (mode != CKM_MODE_DEFER && (!new_centroids || !masses))
        return fail(CKM_ERR_INVALID_ARGUMENT, "new_centroids/masses NULL");
    FusedF32 a{points, old_centroids, labels, new_centroids, masses,
               scratch_view(scratch, scratch_layout(d, k)), n, d, k, mode};
    a.flags = FUSED_BOX_PRUNE | (labels ? 0u : FUSED_NO_LABELS);
    cudaStream_t s = (cudaStream_t)stream;
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::Fused, s);
    return launch_generic_f32(a, Pass::Fused, s);
}

int ckm_labeling_sorted_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, const float* centroids,
                            uint32_t* labels, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (n == 0) return CKM_OK;
    if (!points || !centroids || !labels) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    FusedF32 a{points, centroids, labels, nullptr, nullptr, ScratchView{nullptr, nullptr, nullptr}, n, d, k,
               CKM_MODE_DEFER};
    a.flags = FUSED_BOX_PRUNE;
    cudaStream_t s = (cudaStream_t)stream;
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::LabelOnly, s);
    return launch_generic_f32(a, Pass::LabelOnly, s);
}

size_t ckm_spatial_sort_workspace_bytes(uint64_t n, uint32_t d) { return spatial_sort_workspace_bytes(n, d); }

int ckm_spatial_sort_f32(uint32_t d, uint64_t n, const float* points, float* sorted_points, uint32_t* perm,
                         void* workspace, size_t workspace_bytes, ckm_stream_t stream) {
    if (d == 0 || d > 16) return fail(CKM_ERR_INVALID_ARGUMENT, "spatial sort: num_features must be 1..16");
    if (n > 0xffffffffull) return fail(CKM_ERR_INVALID_ARGUMENT, "spatial sort: num_points must be < 2^32");
    if (n > 0 && (!points || !sorted_points))
        return fail(CKM_ERR_INVALID_ARGUMENT, "spatial sort: NULL pointer");
    if (points == sorted_points && n > 0)
        return fail(CKM_ERR_INVALID_ARGUMENT, "spatial sort: sorted_points must not alias points");
    if (!workspace || workspace_bytes < spatial_sort_workspace_bytes(n, d))
        return fail(CKM_ERR_SCRATCH_TOO_SMALL, "spatial sort: workspace smaller than ckm_spatial_sort_workspace_bytes(n, d)");
    return launch_spatial_sort(d, n, points, sorted_points, perm, workspace, (cudaStream_t)stream);
}

int ckm_unpermute_u32(uint64_t n, const uint32_t* perm, const uint32_t* in, uint32_t* out, ckm_stream_t stream) {
    if (n > 0 && (!perm || !in || !out)) return fail(CKM_ERR_INVALID_ARGUMENT, "unpermute: NULL pointer");
    if (in == out && n > 0) return fail(CKM_ERR_INVALID_ARGUMENT, "unpermute: out must not alias in");
    return launch_unpermute_u32(n, perm, in, out, (cudaStream_t)stream);
}

int ckm_fused_f64(uint32_t d, uint64_t n, uint32_t k, const double* points, const double* old_centroids,
                  double* new_centroids, uint64_t* labels, uint64_t* masses, void* scratch, size_t scratch_bytes,
                  int mode, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (!valid_mode(mode)) return fail(CKM_ERR_INVALID_ARGUMENT, "mode must be DEFER, FINALIZE or ACCUMULATE");
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!old_centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "old_centroids NULL");
    if (mode != CKM_MODE_DEFER && (!new_centroids || !masses))
        return fail(CKM_ERR_INVALID_ARGUMENT, "new_centroids/masses NULL");
    FusedF64 a{points, old_centroids, labels, new_centroids, masses,
               scratch_view(scratch, scratch_layout(d, k)), n, d, k, mode};
    return launch_generic_f64(a, Pass::Fused, (cudaStream_t)stream);
}

int ckm_labeling_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, const float* centroids,
                     uint32_t* labels, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (n == 0) return CKM_OK;
    if (!points || !centroids || !labels) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    FusedF32 a{points, centroids, labels, nullptr, nullptr, ScratchView{nullptr, nullptr, nullptr}, n, d, k,
               CKM_MODE_DEFER};
    cudaStream_t s = (cudaStream_t)stream;
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::LabelOnly, s);
    return launch_generic_f32(a, Pass::LabelOnly, s);
}

int ckm_labeling_f64(uint32_t d, uint64_t n, uint32_t k, const double* points, const double* centroids,
                     uint64_t* labels, ckm_stream_t stream) {
    int st = check_shape(d, n, k);
    if (st) return st;
    if (n == 0) return CKM_OK;
    if (!points || !centroids || !labels) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    FusedF64 a{points, centroids, labels, nullptr, nullptr, ScratchView{nullptr, nullptr, nullptr}, n, d, k,
               CKM_MODE_DEFER};
    return launch_generic_f64(a, Pass::LabelOnly, (cudaStream_t)stream);
}

int ckm_mass_update_u32(uint64_t n, uint32_t k, const uint32_t* labels, uint32_t* masses, ckm_stream_t stream) {
    if (k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters must be >= 1");
    if (n == 0) return CKM_OK;
    if (!labels || !masses) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_mass_u32(n, k, labels, masses, (cudaStream_t)stream);
}

int ckm_mass_update_u64(uint64_t n, uint32_t k, const uint64_t* labels, uint64_t* masses, ckm_stream_t stream) {
    if (k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters must be >= 1");
    if (n == 0) return CKM_OK;
    if (!labels || !masses) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_mass_u64(n, k, labels, masses, (cudaStream_t)stream);
}

int ckm_centroid_update_f32(uint32_t d, uint64_t n, uint32_t k, const float* points, float* centroids,
                            const uint32_t* labels, const uint32_t* masses, void* scratch, size_t scratch_bytes,
                            int mode, ckm_stream_t stream) {
    (void)masses;
    int st = check_shape(d, n, k);
    if (st) return st;
    if (mode != CKM_MODE_DEFER && mode != CKM_MODE_ACCUMULATE)
        return fail(CKM_ERR_INVALID_ARGUMENT, "centroid update mode must be DEFER or ACCUMULATE");
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (mode == CKM_MODE_ACCUMULATE && !centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "centroids NULL");
    FusedF32 a{points, nullptr, const_cast<uint32_t*>(labels), centroids, nullptr,
               scratch_view(scratch, scratch_layout(d, k)), n, d, k, mode};
    cudaStream_t s = (cudaStream_t)stream;
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::SumsOnly, s);
    return launch_generic_f32(a, Pass::SumsOnly, s);
}

int ckm_centroid_update_f64(uint32_t d, uint64_t n, uint32_t k, const double* points, double* centroids,
                            const uint64_t* labels, const uint64_t* masses, void* scratch, size_t scratch_bytes,
                            int mode, ckm_stream_t stream) {
    (void)masses;
    int st = check_shape(d, n, k);
    if (st) return st;
    if (mode != CKM_MODE_DEFER && mode != CKM_MODE_ACCUMULATE)
        return fail(CKM_ERR_INVALID_ARGUMENT, "centroid update mode must be DEFER or ACCUMULATE");
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (mode == CKM_MODE_ACCUMULATE && !centroids) return fail(CKM_ERR_INVALID_ARGUMENT, "centroids NULL");
    FusedF64 a{points, nullptr, const_cast<uint64_t*>(labels), centroids, nullptr,
               scratch_view(scratch, scratch_layout(d, k)), n, d, k, mode};
    return launch_generic_f64(a, Pass::SumsOnly, (cudaStream_t)stream);
}

int ckm_centroid_shift_f32(uint32_t d, uint32_t k, const float* old_c, const float* new_c, float* shift,
                           ckm_stream_t stream) {
    if (d == 0 || k == 0 || !old_c || !new_c || !shift) return fail(CKM_ERR_INVALID_ARGUMENT, "bad shift arguments");
    return launch_shift_f32((uint64_t)k * d, old_c, new_c, shift, (cudaStream_t)stream);
}

int ckm_centroid_shift_f64(uint32_t d, uint32_t k, const double* old_c, const double* new_c, float* shift,
                           ckm_stream_t stream) {
    if (d == 0 || k == 0 || !old_c || !new_c || !shift) return fail(CKM_ERR_INVALID_ARGUMENT, "bad shift arguments");
    return launch_shift_f64((uint64_t)k * d, old_c, new_c, shift, (cudaStream_t)stream);
}

int ckm_matrix_divide_row_f32(uint32_t d, uint32_t k, float* m, const uint32_t* masses, ckm_stream_t stream) {
    if (d == 0 || k == 0 || !m || !masses) return fail(CKM_ERR_INVALID_ARGUMENT, "bad divide arguments");
    return launch_divide_f32(d, k, m, masses, (cudaStream_t)stream);
}

int ckm_matrix_divide_row_f64(uint32_t d, uint32_t k, double* m, const uint64_t* masses, ckm_stream_t stream) {
    if (d == 0 || k == 0 || !m || !masses) return fail(CKM_ERR_INVALID_ARGUMENT, "bad divide arguments");
    return launch_divide_f64(d, k, m, masses, (cudaStream_t)stream);
}

int ckm_matrix_add_f32(uint64_t count, float* a, const float* b, ckm_stream_t stream) {
    if (count == 0) return CKM_OK;
    if (!a || !b) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_add<float>(count, a, b, (cudaStream_t)stream);
}

int ckm_matrix_add_f64(uint64_t count, double* a, const double* b, ckm_stream_t stream) {
    if (count == 0) return CKM_OK;
    if (!a || !b) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_add<double>(count, a, b, (cudaStream_t)stream);
}

int ckm_matrix_add_u32(uint64_t count, uint32_t* a, const uint32_t* b, ckm_stream_t stream) {
    if (count == 0) return CKM_OK;
    if (!a || !b) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_add<uint32_t>(count, a, b, (cudaStream_t)stream);
}

int ckm_matrix_add_u64(uint64_t count, uint64_t* a, const uint64_t* b, ckm_stream_t stream) {
    if (count == 0) return CKM_OK;
    if (!a || !b) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_add<uint64_t>(count, a, b, (cudaStream_t)stream);
}

int ckm_reduce_vector_parcol_u32(uint64_t num_cols, uint64_t num_rows, uint32_t* data, ckm_stream_t stream) {
    if (num_rows == 0 || num_cols == 0) return CKM_OK;
    if (!data) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (num_rows > 0x7fffffffull) return fail(CKM_ERR_INVALID_ARGUMENT, "too many rows");
    return launch_reduce_parcol_u32(num_cols, num_rows, data, (cudaStream_t)stream);
}

int ckm_finalize_f32(uint32_t d, uint32_t k, float* c, uint32_t* m, void* scratch, size_t scratch_bytes,
                     ckm_stream_t stream) {
    int st = check_shape(d, 0, k);
    if (st) return st;
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (!c || !m) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_finalize_f32(d, k, c, m, scratch_view(scratch, scratch_layout(d, k)), CKM_MODE_FINALIZE,
                               (cudaStream_t)stream);
}

int ckm_finalize_f64(uint32_t d, uint32_t k, double* c, uint64_t* m, void* scratch, size_t scratch_bytes,
                     ckm_stream_t stream) {
    int st = check_shape(d, 0, k);
    if (st) return st;
    if ((st = check_scratch(scratch, scratch_bytes, d, k))) return st;
    if (!c || !m) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL pointer");
    return launch_finalize_f64(d, k, c, m, scratch_view(scratch, scratch_layout(d, k)), CKM_MODE_FINALIZE,
                               (cudaStream_t)stream);
}

int ckm_generate_mixture_f32(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed, float clo, float chi,
                             float slo, float shi, uint64_t first, float* points, uint64_t stride,
                             ckm_stream_t stream) {
    if (d == 0 || blobs == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features and num_blobs must be >= 1");
    if (n == 0) return CKM_OK;
    if (!points) return fail(CKM_ERR_INVALID_ARGUMENT, "points NULL");
    if (stride < n) return fail(CKM_ERR_INVALID_ARGUMENT, "points_stride < num_points");
    return launch_generate_f32(d, n, blobs, seed, clo, chi, slo, shi, first, points, stride, (cudaStream_t)stream);
}

}  // extern "C"

extern "C" int ckm_generate_mixture_ex_f32(const ckm_mixture_spec* spec, uint64_t n, uint64_t first, float* points,
                                           uint64_t stride, ckm_stream_t stream) {
    if (!spec) return fail(CKM_ERR_INVALID_ARGUMENT, "spec is NULL");
    if (spec->num_features == 0 || spec->num_blobs == 0)
        return fail(CKM_ERR_INVALID_ARGUMENT, "num_features and num_blobs must be >= 1");
    if (spec->sigma_dist && !(spec->sigma_lo > 0.0f && spec->sigma_hi > 0.0f))
        return fail(CKM_ERR_INVALID_ARGUMENT, "log-uniform sigma needs positive bounds");
    if (n == 0) return CKM_OK;
    if (!points) return fail(CKM_ERR_INVALID_ARGUMENT, "points NULL");
    if (stride < n) return fail(CKM_ERR_INVALID_ARGUMENT, "points_stride < num_points");
    return launch_generate_ex_f32(spec->num_features, n, spec->num_blobs, spec->seed, spec->center_dist,
                                  spec->center_a, spec->center_b, spec->sigma_dist, spec->sigma_lo, spec->sigma_hi,
                                  spec->dirichlet, first, points, stride, (cudaStream_t)stream);
}
