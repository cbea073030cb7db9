// ckm_fused_f32_noalloc: the fused Lloyd iteration for callers that cannot
// allocate device memory.
//
// Some callers have no way to obtain a scratch buffer. Examples: a plugin
// that runs inside a host framework which owns every byte of device memory
// and forbids allocation from its callbacks; a latency-critical loop that
// must never hit cudaMalloc/cudaFree (cudaFree waits for the whole device);
// an embedded caller that was handed only the input and output buffers.
// This entry point needs nothing from them but those buffers: the FP64
// merge scratch that ckm_fused_f32 takes as an argument lives here in a
// fixed, file-scope device array instead.
//
// Costs of that choice, stated for the user:
//   - the array (NOALLOC_SCRATCH_BYTES = 128 KiB) exists on every GPU that
//     loads this library, for as long as the process runs;
//   - it bounds the problem size: ckm_scratch_bytes(d, k) must fit in it
//     (about k*d <= 15,000; e.g. k = 1024 with d = 8, k = 16 with d = 512);
//     larger sizes are rejected with CKM_ERR_SCRATCH_TOO_SMALL;
//   - every call on a device shares the one array, so calls that can run at
//     the same time on the GPU (different streams, other threads) race and
//     corrupt each other's sums: order them on one stream or serialize them;
//   - the array keeps the previous call's contents, so each call clears the
//     part it uses (one cudaMemsetAsync on the caller's stream) before the
//     kernel runs.
// Set-up: the first call in each CUDA context (the first call on each device,
// and the first one again after cudaDeviceReset or after a driver-API caller
// made another context current) looks up the array's device address with
// that device current (cudaGetSymbolAddress, which also loads this module);
// later calls in the same context reuse it.  Make that first call before any
// stream capture begins.
#include <cuda.h>

#include <mutex>

#include "ckm_internal.h"

namespace ckm {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 128 * 1024;
constexpr int MAX_DEVICES = 64;

// The built-in scratch.  Host code must not use this name as an address: it
// is a host-side shadow.  The device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
void* g_scratch_addr[MAX_DEVICES];
unsigned long long g_scratch_ctx[MAX_DEVICES];  // id of the context the address belongs to (0: none)

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Process-unique id of the current CUDA context (cuCtxGetId, reached through
// the runtime's driver entry points, so the library needs no -lcuda); 0 when
// no context is current or the entry points are unavailable.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_cur || !get_id) return 0;
    CUcontext c = nullptr;
    if (get_cur(&c) != CUDA_SUCCESS || !c) return 0;
    unsigned long long id = 0;
    return get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of the built-in scratch in the current context: looked up
// once per context (a cached address from a context that was reset or is not
// current any more would point at memory this call does not own).
int builtin_scratch(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= MAX_DEVICES) return fail(CKM_ERR_UNSUPPORTED, "device ordinal out of range");
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> g(g_mu);
    if (ctx == 0 || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(built-in scratch)");
        if (p == nullptr) return fail(CKM_ERR_CUDA, "built-in scratch has no device address");
        g_scratch_addr[dev] = p;
        // the lookup made the device's primary context current if none was
        g_scratch_ctx[dev] = ctx ? ctx : current_context_id();
    }
    *out = g_scratch_addr[dev];
    return CKM_OK;
}

}  // namespace
}  // namespace ckm

using namespace ckm;

extern "C" int ckm_fused_f32_noalloc(uint32_t d, uint64_t n, uint32_t k, const float* points,
                                     const float* old_centroids, float* new_centroids, uint32_t* labels,
                                     uint32_t* masses, int mode, ckm_stream_t stream) {
    if (d == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_features must be >= 1");
    if (k == 0) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters must be >= 1");
    if (mode != CKM_MODE_FINALIZE && mode != CKM_MODE_ACCUMULATE)
        return fail(CKM_ERR_INVALID_ARGUMENT,
                    "ckm_fused_f32_noalloc: mode must be FINALIZE or ACCUMULATE (DEFER would keep sums in the "
                    "shared built-in scratch between calls)");
    if ((uint64_t)k * d > (1ull << 31)) return fail(CKM_ERR_INVALID_ARGUMENT, "num_clusters * num_features too large");
    const ScratchLayout L = scratch_layout(d, k);
    if (L.total > NOALLOC_SCRATCH_BYTES)
        return fail(CKM_ERR_SCRATCH_TOO_SMALL,
                    "ckm_fused_f32_noalloc: this (num_features, num_clusters) needs " + std::to_string(L.total) +
                        " bytes of scratch; the built-in scratch holds " + std::to_string(NOALLOC_SCRATCH_BYTES) +
                        " bytes. Use ckm_fused_f32 with caller-provided scratch instead.");
    if (n > 0 && (!points || !labels)) return fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!old_centroids || !new_centroids || !masses)
        return fail(CKM_ERR_INVALID_ARGUMENT, "old_centroids/new_centroids/masses NULL");

    void* base = nullptr;
    int st = builtin_scratch(&base);
    if (st != CKM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // the previous call left its data behind: clear the part this call uses
    cudaError_t e = cudaMemsetAsync(base, 0, L.total, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(built-in scratch)");
    FusedF32 a{points, old_centroids, labels, new_centroids, masses, scratch_view(base, L), n, d, k, mode};
    if (lowd_supported(d, k)) return launch_fused_f32(a, Pass::Fused, s);
    return launch_generic_f32(a, Pass::Fused, s);
}
