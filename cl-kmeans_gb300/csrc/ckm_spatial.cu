// Spatial order for the low-d fused kernel's box pruning.
//
// A stable LSD radix sort of the points by a 16-bit Z-order (Morton) key of
// their cells: each feature's range [min, max] is cut into 2^b bins
// (b = max(1, 16 / d) for d <= 16), and the bins' bits interleave into the
// key, so consecutive keys are neighbouring cells.  After the sort every
// 256-point warp tile of the fused kernel covers one or a few small cells, and
// most clusters are provably farther than another from all of its points
// (FUSED_BOX_PRUNE).  The sort is a layout of the caller's point set, not part
// of the arithmetic: labels computed on the sorted set go back to the caller's
// order through the permutation (unpermute).
//
//   bbox:      per-feature min / max (order-preserving integer atomics)
//   per pass (8 key bits, low byte first; the key is recomputed from the
//   point, and the points and their original indices travel with it):
//   upsweep:   per chunk (CHUNK consecutive items), the count of each digit
//   scan:      exclusive prefix of the counts in digit-major order: where each
//              (digit, chunk) run starts in the output
//   downsweep: each CTA ranks its chunk's items by digit, stably, in shared
//              memory (rounds of 256 items, warp match + per-warp counts), and
//              writes each digit's run contiguously (coalesced), gathering
//              the points from the chunk it has just read
#include <cuda_runtime.h>

#include "ckm_device.cuh"
#include "ckm_internal.h"

namespace ckm {
namespace {

constexpr int SB = 256;

__device__ __forceinline__ uint32_t ord_of(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float float_of(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Workspace: [0, 16) min (ordered), [16, 32) max (ordered), the counts /
// offsets [RADIX * chunks], the scan's block sums, then the intermediate
// points [d * n] and indices [n] between the two passes.
constexpr uint32_t RADIX = 256;
constexpr uint32_t SCAN_PER_BLOCK = 4096;

struct SortWs {
    uint32_t* lo;
    uint32_t* hi;
    uint32_t* counts;
    uint32_t* block_sums;
    float* tmp_points;
    uint32_t* tmp_idx;
};

// Items per chunk: the chunk is re-read (gathered) from L2 when written out, so
// it stays a 64 KiB window of points.
uint32_t chunk_items(uint32_t d) { return d <= 4 ? 4096u : (d <= 8 ? 2048u : 1024u); }

uint64_t num_chunks(uint64_t n, uint32_t d) { return (n + chunk_items(d) - 1) / chunk_items(d); }

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

uint64_t scan_blocks_of(uint64_t n, uint32_t d) {
    return ((uint64_t)RADIX * num_chunks(n, d) + SCAN_PER_BLOCK - 1) / SCAN_PER_BLOCK;
}

SortWs sort_ws(void* ws, uint64_t n, uint32_t d) {
    unsigned char* w = static_cast<unsigned char*>(ws);
    const size_t counts = a256((size_t)RADIX * num_chunks(n, d) * 4);
    const size_t sums = a256((size_t)scan_blocks_of(n, d) * 4);
    SortWs r;
    r.lo = reinterpret_cast<uint32_t*>(w);
    r.hi = r.lo + 16;
    r.counts = reinterpret_cast<uint32_t*>(w + 256);
    r.block_sums = reinterpret_cast<uint32_t*>(w + 256 + counts);
    r.tmp_points = reinterpret_cast<float*>(w + 256 + counts + sums);
    r.tmp_idx = reinterpret_cast<uint32_t*>(w + 256 + counts + sums + a256((size_t)n * d * 4));
    return r;
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

// Digit (8 bits at `shift`) of item i of a pass's input.
__device__ __forceinline__ uint32_t item_digit(const float* __restrict__ P, uint64_t n, uint64_t i, uint32_t d,
                                               uint32_t b, const float* lo, const float* scale, uint32_t shift) {
    return (point_key(P, n, i, d, b, lo, scale) >> shift) & (RADIX - 1u);
}

// Digit histogram of one chunk into s_hist (warp-aggregated shared atomics);
// every thread of the CTA calls it.
__device__ __forceinline__ void chunk_histogram(const float* __restrict__ P, uint64_t n, uint32_t d, uint32_t b,
                                                const float* lo, const float* scale, uint32_t shift, uint64_t c0,
                                                uint32_t chunk, uint32_t* s_hist) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t j = threadIdx.x; j < RADIX; j += SB) s_hist[j] = 0u;
    __syncthreads();
    for (uint32_t r = 0; r < chunk; r += SB) {
        const uint64_t i = c0 + r + threadIdx.x;
        const bool ok = i < n;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const uint32_t dg = item_digit(P, n, i, d, b, lo, scale, shift);
            const uint32_t peers = __match_any_sync(active, dg);
            if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&s_hist[dg], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(SB) upsweep_kernel(const float* __restrict__ P, uint64_t n, uint32_t d, uint32_t b,
                                                     SortWs ws, uint32_t shift, uint32_t chunk, uint64_t chunks) {
    __shared__ uint32_t s_hist[RADIX];
    float lo[16], scale[16];
    load_range(ws, d, b, lo, scale);
    const uint64_t c = blockIdx.x;
    chunk_histogram(P, n, d, b, lo, scale, shift, c * chunk, chunk, s_hist);
    for (uint32_t j = threadIdx.x; j < RADIX; j += SB) ws.counts[(uint64_t)j * chunks + c] = s_hist[j];
}

// Exclusive scan of counts[0, m) in place: block sums, then their scan, then
// each block's prefix.
__global__ void __launch_bounds__(SB) scan_sums_kernel(const uint32_t* __restrict__ v, uint64_t m, uint32_t* sums) {
    __shared__ uint32_t s_w[SB / 32];
    const uint64_t b0 = (uint64_t)blockIdx.x * SCAN_PER_BLOCK;
    uint32_t t = 0;
    for (uint32_t j = threadIdx.x; j < SCAN_PER_BLOCK; j += SB)
        if (b0 + j < m) t += v[b0 + j];
    t = __reduce_add_sync(0xffffffffu, t);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < SB / 32; ++w) s += s_w[w];
        sums[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(1024) scan_block_sums_kernel(uint32_t* sums, uint32_t nb) {
    // exclusive scan of nb values: each thread a run of ceil(nb / 1024)
    __shared__ uint32_t s_part[1024];
    const uint32_t t = threadIdx.x;
    const uint32_t per = (nb + 1023u) / 1024u;
    const uint32_t j0 = t * per;
    uint32_t tot = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (j0 + i < nb) tot += sums[j0 + i];
    s_part[t] = tot;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1) {
        const uint32_t x = t >= o ? s_part[t - o] : 0u;
        __syncthreads();
        s_part[t] += x;
        __syncthreads();
    }
    uint32_t run = s_part[t] - tot;
    for (uint32_t i = 0; i < per; ++i)
        if (j0 + i < nb) {
            const uint32_t v = sums[j0 + i];
            sums[j0 + i] = run;
            run += v;
        }
}

__global__ void __launch_bounds__(SB) scan_apply_kernel(uint32_t* v, uint64_t m, const uint32_t* __restrict__ sums) {
    // per block: 16 consecutive values per thread, a block scan of the
    // thread totals, plus the block's offset
    __shared__ uint32_t s_part[SB];
    const uint64_t b0 = (uint64_t)blockIdx.x * SCAN_PER_BLOCK;
    const uint32_t per = SCAN_PER_BLOCK / SB;
    const uint64_t j0 = b0 + (uint64_t)threadIdx.x * per;
    uint32_t x[SCAN_PER_BLOCK / SB], tot = 0;
    for (uint32_t i = 0; i < per; ++i) {
        x[i] = j0 + i < m ? v[j0 + i] : 0u;
        tot += x[i];
    }
    s_part[threadIdx.x] = tot;
    __syncthreads();
    for (uint32_t o = 1; o < SB; o <<= 1) {
        const uint32_t y = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0u;
        __syncthreads();
        s_part[threadIdx.x] += y;
        __syncthreads();
    }
    uint32_t run = sums[blockIdx.x] + s_part[threadIdx.x] - tot;
    for (uint32_t i = 0; i < per; ++i) {
        if (j0 + i < m) v[j0 + i] = run;
        run += x[i];
    }
}

// One pass's scatter for one chunk:
//   1. the chunk's items are read once (coalesced); their digits go to shared
//      memory and into the chunk's histogram;
//   2. the items are ranked stably within their digits in rounds of SB (item
//      order = round, then thread; warp match + per-warp counts), entirely in
//      shared memory: s_src[pos] = the chunk-local index of the item at
//      position pos of the chunk sorted by digit;
//   3. the sorted chunk is written out digit run by digit run (consecutive
//      output positions, coalesced), gathering the point values from the
//      chunk just read (an L2-resident window).
__global__ void __launch_bounds__(SB) downsweep_kernel(const float* __restrict__ P, const uint32_t* __restrict__ idx_in,
                                                       uint64_t n, uint32_t d, uint32_t b, SortWs ws, uint32_t shift,
                                                       uint32_t chunk, uint64_t chunks, float* __restrict__ P_out,
                                                       uint32_t* __restrict__ idx_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint16_t* s_src = reinterpret_cast<uint16_t*>(smem);                 // [chunk]
    unsigned char* s_din = reinterpret_cast<unsigned char*>(s_src + chunk);  // digit of local item j
    unsigned char* s_dig = s_din + chunk;                                 // digit at sorted position
    constexpr uint32_t NW = SB / 32;
    // per warp and digit: the warp's count, then the absolute position of its
    // next item of that digit
    __shared__ uint32_t s_off[RADIX], s_wh[NW][RADIX], s_ws[NW];
    float lo[16], scale[16];
    load_range(ws, d, b, lo, scale);
    const uint64_t c = blockIdx.x;
    const uint64_t c0 = c * chunk;
    const uint32_t valid = (uint32_t)min((uint64_t)chunk, n - c0);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // each warp owns a contiguous run of the chunk's items (chunk is a
    // multiple of SB), so only warp-level synchronisation is needed while
    // digits are counted and positions handed out; the warps' runs in order
    // keep the sort stable
    const uint32_t per = chunk / NW, w0 = warp * per;

    // 1. digits and per-warp histograms
    for (uint32_t t = lane; t < RADIX; t += 32) s_wh[warp][t] = 0u;
    __syncwarp();
    for (uint32_t r = 0; r < per; r += 32) {
        const uint32_t j = w0 + r + lane;
        const bool ok = j < valid;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const uint32_t dg = item_digit(P, n, c0 + j, d, b, lo, scale, shift);
            s_din[j] = (unsigned char)dg;
            const uint32_t peers = __match_any_sync(active, dg);
            if (lane == (uint32_t)(__ffs(peers) - 1)) s_wh[warp][dg] += (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // 2. thread t = digit t (SB == RADIX): the counts of the warps before each
    // warp, the digit's total, and the exclusive scan of the totals
    {
        const uint32_t t = threadIdx.x;
        uint32_t tot = 0;
        for (uint32_t w = 0; w < NW; ++w) {
            const uint32_t v = s_wh[w][t];
            s_wh[w][t] = tot;
            tot += v;
        }
        uint32_t incl = tot;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_ws[warp] = incl;
        __syncthreads();
        uint32_t base = 0;
        for (uint32_t w = 0; w < warp; ++w) base += s_ws[w];
        const uint32_t excl = base + incl - tot;
        s_off[t] = excl;
        for (uint32_t w = 0; w < NW; ++w) s_wh[w][t] += excl;
    }
    __syncthreads();

    // 3. stable positions: each warp hands out positions to its items in order
    for (uint32_t r = 0; r < per; r += 32) {
        const uint32_t j = w0 + r + lane;
        const bool ok = j < valid;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        if (ok) {
            const uint32_t dg = s_din[j];
            const uint32_t peers = __match_any_sync(active, dg);
            const uint32_t pos = s_wh[warp][dg] + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            s_src[pos] = (uint16_t)j;
            s_dig[pos] = (unsigned char)dg;
            __syncwarp(active);  // every lane has read its base before the leader moves it
            if (lane == (uint32_t)(__ffs(peers) - 1)) s_wh[warp][dg] += (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // 3. write out
    for (uint32_t q = threadIdx.x; q < valid; q += SB) {
        const uint32_t dg = s_dig[q];
        const uint32_t src = s_src[q];
        const uint64_t g = (uint64_t)ws.counts[(uint64_t)dg * chunks + c] + (q - s_off[dg]);
        for (uint32_t f = 0; f < d; ++f) P_out[(size_t)f * n + g] = __ldg(P + (size_t)f * n + c0 + src);
        idx_out[g] = idx_in ? __ldg(idx_in + c0 + src) : (uint32_t)(c0 + src);
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

size_t spatial_sort_workspace_bytes(uint64_t n, uint32_t d) {
    if (d == 0) return 0;
    return 256 + a256((size_t)RADIX * num_chunks(n, d) * 4) + a256((size_t)scan_blocks_of(n, d) * 4) +
           a256((size_t)n * d * 4) + a256((size_t)n * 4);
}

namespace {
size_t downsweep_smem(uint32_t d) { return (size_t)chunk_items(d) * 4; }  // s_src (u16) + two digit arrays
}  // namespace

int launch_spatial_sort(uint32_t d, uint64_t n, const float* points, float* sorted, uint32_t* perm, void* ws_ptr,
                        cudaStream_t s) {
    SortWs ws = sort_ws(ws_ptr, n, d);
    // lo = all ones (min identity), hi = zero
    cudaError_t e = cudaMemsetAsync(ws.lo, 0xff, 16 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ws.hi, 0, 16 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_fail(e, "spatial sort: workspace init");
    if (n == 0) return CKM_OK;
    const uint32_t b = d >= 16 ? 1u : 16u / d;
    const uint32_t chunk = chunk_items(d);
    const uint64_t chunks = num_chunks(n, d);
    const uint64_t m = (uint64_t)RADIX * chunks;
    const uint64_t scan_blocks = scan_blocks_of(n, d);
    const size_t smem = downsweep_smem(d);
    static bool attr_done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, downsweep_kernel);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(spatial downsweep)");
        e = cudaFuncSetAttribute(downsweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(device_info().smem_optin - fa.sharedSizeBytes));
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(spatial downsweep)");
        attr_done[dev] = true;
    }
    bbox_kernel<<<grid_of(n), SB, 0, s>>>(points, n, d, ws);
    for (uint32_t pass = 0; pass < 2; ++pass) {
        const uint32_t shift = 8 * pass;
        const float* src = pass == 0 ? points : ws.tmp_points;
        const uint32_t* src_idx = pass == 0 ? nullptr : ws.tmp_idx;
        float* dst = pass == 0 ? ws.tmp_points : sorted;
        uint32_t* dst_idx = pass == 0 ? ws.tmp_idx : perm;
        upsweep_kernel<<<(unsigned)chunks, SB, 0, s>>>(src, n, d, b, ws, shift, chunk, chunks);
        scan_sums_kernel<<<(unsigned)scan_blocks, SB, 0, s>>>(ws.counts, m, ws.block_sums);
        scan_block_sums_kernel<<<1, 1024, 0, s>>>(ws.block_sums, (uint32_t)scan_blocks);
        scan_apply_kernel<<<(unsigned)scan_blocks, SB, 0, s>>>(ws.counts, m, ws.block_sums);
        downsweep_kernel<<<(unsigned)chunks, SB, smem, s>>>(src, src_idx, n, d, b, ws, shift, chunk, chunks, dst,
                                                            dst_idx);
    }
    count_launch(11);
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
