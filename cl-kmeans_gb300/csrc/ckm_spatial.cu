// Spatial order for the low-d fused kernel's box pruning.
//
// A counting sort of the points by a 16-bit Z-order (Morton) key of their
// cells: each feature's range [min, max] is cut into 2^b bins
// (b = max(1, 16 / d) for d <= 16), and the bins' bits interleave into the
// key, so consecutive keys are neighbouring cells.  After the sort every
// 256-point warp tile of the fused kernel covers one or a few small cells, and
// most clusters are provably farther than another from all of its points
// (FUSED_BOX_PRUNE).  The sort is a layout of the caller's point set, not part
// of the arithmetic: labels computed on the sorted set go back to the caller's
// order through the permutation (unpermute).
//
//   bbox:    per-feature min / max (order-preserving integer atomics)
//   count:   points per key (warp-aggregated global atomics)
//   scan:    exclusive prefix of the 65536 counts (one CTA)
//   scatter: position = start of the key + running count (warp-aggregated),
//            sorted[f * n + pos] = points[f * n + p], perm[pos] = p
#include <cuda_runtime.h>

#include "ckm_device.cuh"
#include "ckm_internal.h"

namespace ckm {
namespace {

constexpr uint32_t KEY_BINS = 1u << 16;
constexpr int SB = 256;

__device__ __forceinline__ uint32_t ord_of(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float float_of(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// ws layout: [0, 16) min (ordered), [16, 32) max (ordered), then counts
// [KEY_BINS], then cursors [KEY_BINS].
struct SortWs {
    uint32_t* lo;
    uint32_t* hi;
    uint32_t* counts;
    uint32_t* cursor;
};

SortWs sort_ws(void* ws) {
    uint32_t* w = static_cast<uint32_t*>(ws);
    return SortWs{w, w + 16, w + 32, w + 32 + KEY_BINS};
}

__global__ void __launch_bounds__(SB) bbox_kernel(const float* __restrict__ P, uint64_t n, uint32_t d, SortWs ws) {
    __shared__ uint32_t s_lo[16], s_hi[16];
    if (threadIdx.x < 16) {
        s_lo[threadIdx.x] = 0xffffffffu;
        s_hi[threadIdx.x] = 0u;
    }
    __syncthreads();
    for (uint32_t f = 0; f < d; ++f) {
        float lo = INFINITY, hi = -INFINITY;
        for (uint64_t p = (uint64_t)blockIdx.x * SB + threadIdx.x; p < n; p += (uint64_t)gridDim.x * SB) {
            const float v = __ldg(P + (size_t)f * n + p);
            lo = fminf(lo, v);  // NaN ignored
            hi = fmaxf(hi, v);
        }
        const uint32_t ol = __reduce_min_sync(0xffffffffu, ord_of(lo));
        const uint32_t oh = __reduce_max_sync(0xffffffffu, ord_of(hi));
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&s_lo[f], ol);
            atomicMax(&s_hi[f], oh);
        }
    }
    __syncthreads();
    if (threadIdx.x < d) {
        atomicMin(&ws.lo[threadIdx.x], s_lo[threadIdx.x]);
        atomicMax(&ws.hi[threadIdx.x], s_hi[threadIdx.x]);
    }
}

// Z-order key of point p (b bits per feature, d * b <= 16).
__device__ __forceinline__ uint32_t point_key(const float* __restrict__ P, uint64_t n, uint64_t p, uint32_t d,
                                              uint32_t b, const float* lo, const float* scale) {
    const uint32_t top = (1u << b) - 1u;
    uint32_t key = 0;
    for (uint32_t f = 0; f < d; ++f) {
        const float v = (__ldg(P + (size_t)f * n + p) - lo[f]) * scale[f];
        // NaN and values below the range go to bin 0, above it to the top bin
        const uint32_t q = v >= (float)top ? top : (v >= 1.0f ? (uint32_t)v : 0u);
        for (uint32_t i = 0; i < b; ++i) key |= ((q >> i) & 1u) << (i * d + f);
    }
    return key;
}

__device__ __forceinline__ void load_range(const SortWs& ws, uint32_t d, uint32_t b, float* lo, float* scale) {
    for (uint32_t f = 0; f < d; ++f) {
        const float l = float_of(ws.lo[f]), h = float_of(ws.hi[f]);
        lo[f] = l;
        const float w = h - l;
        scale[f] = (w > 0.0f && w < INFINITY) ? (float)(1u << b) / w : 0.0f;
        if (!(l > -INFINITY && l < INFINITY)) lo[f] = 0.0f;
    }
}

__global__ void __launch_bounds__(SB) count_kernel(const float* __restrict__ P, uint64_t n, uint32_t d, uint32_t b,
                                                   SortWs ws) {
    float lo[16], scale[16];
    load_range(ws, d, b, lo, scale);
    const uint32_t lane = threadIdx.x & 31u;
    for (uint64_t base = (uint64_t)blockIdx.x * SB + (threadIdx.x & ~31u); base < n; base += (uint64_t)gridDim.x * SB) {
        const uint64_t p = base + lane;
        const bool ok = p < n;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        if (!ok) continue;
        const uint32_t key = point_key(P, n, p, d, b, lo, scale);
        const uint32_t peers = __match_any_sync(active, key);
        if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&ws.counts[key], (uint32_t)__popc(peers));
    }
}

__global__ void __launch_bounds__(1024) scan_kernel(SortWs ws) {
    // 65536 counts, 64 per thread: exclusive prefix into cursor
    __shared__ uint32_t s_part[1024];
    const uint32_t t = threadIdx.x;
    uint32_t sum = 0;
    for (uint32_t i = 0; i < 64; ++i) sum += ws.counts[t * 64 + i];
    s_part[t] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1) {
        const uint32_t v = t >= o ? s_part[t - o] : 0u;
        __syncthreads();
        s_part[t] += v;
        __syncthreads();
    }
    uint32_t run = s_part[t] - sum;  // exclusive
    for (uint32_t i = 0; i < 64; ++i) {
        ws.cursor[t * 64 + i] = run;
        run += ws.counts[t * 64 + i];
    }
}

__global__ void __launch_bounds__(SB) scatter_kernel(const float* __restrict__ P, uint64_t n, uint32_t d, uint32_t b,
                                                     SortWs ws, float* __restrict__ out, uint32_t* __restrict__ perm) {
    float lo[16], scale[16];
    load_range(ws, d, b, lo, scale);
    const uint32_t lane = threadIdx.x & 31u;
    for (uint64_t base = (uint64_t)blockIdx.x * SB + (threadIdx.x & ~31u); base < n; base += (uint64_t)gridDim.x * SB) {
        const uint64_t p = base + lane;
        const bool ok = p < n;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        if (!ok) continue;
        const uint32_t key = point_key(P, n, p, d, b, lo, scale);
        const uint32_t peers = __match_any_sync(active, key);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t start = 0;
        if (lane == leader) start = atomicAdd(&ws.cursor[key], (uint32_t)__popc(peers));
        start = __shfl_sync(peers, start, leader);
        const uint32_t pos = start + __popc(peers & ((1u << lane) - 1u));
        for (uint32_t f = 0; f < d; ++f) out[(size_t)f * n + pos] = __ldg(P + (size_t)f * n + p);
        perm[pos] = (uint32_t)p;
    }
}

__global__ void __launch_bounds__(SB) unpermute_kernel(uint64_t n, const uint32_t* __restrict__ perm,
                                                       const uint32_t* __restrict__ in, uint32_t* __restrict__ out) {
    for (uint64_t q = (uint64_t)blockIdx.x * SB + threadIdx.x; q < n; q += (uint64_t)gridDim.x * SB)
        out[perm[q]] = in[q];
}

uint32_t grid_of(uint64_t n) {
    uint64_t g = (n + SB - 1) / SB;
    const uint64_t cap = (uint64_t)device_info().sm_count * 8;
    if (g > cap) g = cap;
    return (uint32_t)(g < 1 ? 1 : g);
}

}  // namespace

size_t spatial_sort_workspace_bytes() { return (32 + 2 * (size_t)KEY_BINS) * sizeof(uint32_t); }

int launch_spatial_sort(uint32_t d, uint64_t n, const float* points, float* sorted, uint32_t* perm, void* ws_ptr,
                        cudaStream_t s) {
    SortWs ws = sort_ws(ws_ptr);
    // lo = all ones (min identity), hi and the counts = zero
    cudaError_t e = cudaMemsetAsync(ws.lo, 0xff, 16 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ws.hi, 0, (16 + 2 * (size_t)KEY_BINS) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_fail(e, "spatial sort: workspace init");
    if (n == 0) return CKM_OK;
    const uint32_t b = d >= 16 ? 1u : 16u / d;
    const uint32_t g = grid_of(n);
    bbox_kernel<<<g, SB, 0, s>>>(points, n, d, ws);
    count_kernel<<<g, SB, 0, s>>>(points, n, d, b, ws);
    scan_kernel<<<1, 1024, 0, s>>>(ws);
    scatter_kernel<<<g, SB, 0, s>>>(points, n, d, b, ws, sorted, perm);
    count_launch(4);
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "spatial sort launch");
}

int launch_unpermute_u32(uint64_t n, const uint32_t* perm, const uint32_t* in, uint32_t* out, cudaStream_t s) {
    if (n == 0) return CKM_OK;
    unpermute_kernel<<<grid_of(n), SB, 0, s>>>(n, perm, in, out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "unpermute launch");
}

}  // namespace ckm
