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
// The pipeline moves each point a minimal number of times (at n = 2^28,
// d = 4: two reads and two writes of the 4 GiB of points, plus 2-byte keys):
//   bbox:     per-feature min / max over a strided sample of 2^20 points
//             (points outside the sample's range fall in the edge cells);
//   keys:     one pass over the points: the 16-bit key of every point into a
//             padded key array, and per chunk of CH consecutive points the
//             histogram of the key's low byte;
//   scan:     exclusive prefix of the chunk histograms in digit-major order
//             (where each (digit, chunk) run starts in the output), stored
//             chunk-major so a chunk reads its 256 offsets in one 1 KiB row;
//   scatter:  per chunk, the keys and then the points (and indices) are
//             staged in shared memory by cp.async; while the points are in
//             flight the chunk's items are ranked stably within their digits
//             (warps own contiguous runs of items; warp match + per-warp
//             counts; one pass); then every digit's run is written out
//             contiguously (coalesced), reading the staged points;
//   pass 2:   the histogram of the high byte over the pass-1 keys (2 bytes a
//             point), the scan, and the same scatter on the high byte.
#include <cuda_runtime.h>

#include <algorithm>

#include "ckm_device.cuh"
#include "ckm_internal.h"

namespace ckm {
namespace {

constexpr int SB = 512;                      // threads per CTA: key, histogram and scatter kernels
constexpr uint32_t RADIX = 256;
constexpr uint32_t BBOX_SAMPLES = 1u << 20;  // points sampled for the bounding box
constexpr uint32_t SCAN_ROWS = 256;          // chunks per block of the offset scan
constexpr uint32_t SCAN_BATCH = 16;          // independent rows loaded together in the scan

__device__ __forceinline__ uint32_t ord_of(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float float_of(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Points per chunk: a chunk's staged points are 64 KiB for every d (4096
// points for d <= 4).  512-thread CTAs, two per SM, rank and write a chunk
// each (a 256-thread shape on half the chunk measured 20 % slower).
__host__ __device__ constexpr uint32_t chunk_of(uint32_t d) { return 4096u / (d <= 4 ? 1u : (d <= 8 ? 2u : 4u)); }
uint32_t chunk_items(uint32_t d) { return chunk_of(d); }
uint64_t num_chunks(uint64_t n, uint32_t d) { return (n + chunk_items(d) - 1) / chunk_items(d); }
uint64_t scan_blocks_of(uint64_t chunks) { return (chunks + SCAN_ROWS - 1) / SCAN_ROWS; }
size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

// Workspace: [0, 64) min (ordered), [64, 128) max (ordered); the chunk
// offsets [chunks][RADIX]; the scan's block partials [blocks + 1][RADIX]; two
// padded key arrays [chunks * CH]; the points [d * n] and indices [n] between
// the two passes.
struct SortWs {
    uint32_t* lo;
    uint32_t* hi;
    uint32_t* counts;
    uint32_t* partial;
    uint16_t* keys0;
    uint16_t* keys1;
    float* tmp_points;
    uint32_t* tmp_idx;
};

struct WsSizes {
    size_t counts, partial, keys, pts, idx;
};
WsSizes ws_sizes(uint64_t n, uint32_t d) {
    WsSizes z;
    const uint64_t ch = chunk_of(d), chunks = (n + ch - 1) / ch;
    z.counts = a256((size_t)RADIX * chunks * 4);
    z.partial = a256((size_t)RADIX * (scan_blocks_of(chunks) + 1) * 4);
    z.keys = a256((size_t)chunks * ch * 2);
    z.pts = a256((size_t)n * d * 4);
    z.idx = a256((size_t)n * 4);
    return z;
}

SortWs sort_ws(void* ws, uint64_t n, uint32_t d) {
    unsigned char* w = static_cast<unsigned char*>(ws);
    const WsSizes z = ws_sizes(n, d);
    SortWs r;
    size_t off = 256;
    r.lo = reinterpret_cast<uint32_t*>(w);
    r.hi = r.lo + 16;
    r.counts = reinterpret_cast<uint32_t*>(w + off);
    off += z.counts;
    r.partial = reinterpret_cast<uint32_t*>(w + off);
    off += z.partial;
    r.keys0 = reinterpret_cast<uint16_t*>(w + off);
    off += z.keys;
    r.keys1 = reinterpret_cast<uint16_t*>(w + off);
    off += z.keys;
    r.tmp_points = reinterpret_cast<float*>(w + off);
    off += z.pts;
    r.tmp_idx = reinterpret_cast<uint32_t*>(w + off);
    return r;
}

// --- cp.async (per-thread asynchronous global -> shared copies) ------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Copies count 32-bit words src[0, count) to dst (shared) with 16-byte copies
// where both sides allow it (vec: src 16-byte aligned), 4-byte ones for the
// rest; every thread of the CTA takes part.
template <int BT>
__device__ __forceinline__ void stage_words(uint32_t* dst, const uint32_t* src, uint32_t count, bool vec) {
    uint32_t done = 0;
    if (vec) {
        const uint32_t nv = count / 4;
        for (uint32_t i = threadIdx.x; i < nv; i += BT) cp_async16(dst + 4 * i, src + 4 * i);
        done = nv * 4;
    }
    for (uint32_t i = done + threadIdx.x; i < count; i += BT) cp_async4(dst + i, src + i);
}

// --- bounding box from a strided sample ------------------------------------
__global__ void __launch_bounds__(256) bbox_sample_kernel(const float* __restrict__ P, uint64_t n, uint32_t d,
                                                          uint64_t stride, uint32_t samples, uint32_t* lo_out,
                                                          uint32_t* hi_out) {
    __shared__ uint32_t s_lo[16], s_hi[16];
    if (threadIdx.x < 16) {
        s_lo[threadIdx.x] = 0xffffffffu;
        s_hi[threadIdx.x] = 0u;
    }
    __syncthreads();
    for (uint32_t f = 0; f < d; ++f) {
        float lo = INFINITY, hi = -INFINITY;
        for (uint32_t i = blockIdx.x * 256u + threadIdx.x; i < samples; i += gridDim.x * 256u) {
            const float v = __ldg(P + (size_t)f * n + (uint64_t)i * stride);
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
        atomicMin(&lo_out[threadIdx.x], s_lo[threadIdx.x]);
        atomicMax(&hi_out[threadIdx.x], s_hi[threadIdx.x]);
    }
}

// Bin origin and scale of each feature (threads < d; into shared memory).
__device__ __forceinline__ void load_range(const uint32_t* lo_w, const uint32_t* hi_w, uint32_t d, uint32_t b,
                                           float* s_lo, float* s_scale) {
    if (threadIdx.x < d) {
        const uint32_t f = threadIdx.x;
        const float l = float_of(lo_w[f]), h = float_of(hi_w[f]);
        const float w = h - l;
        s_scale[f] = (w > 0.0f && w < INFINITY) ? (float)(1u << b) / w : 0.0f;
        s_lo[f] = (l > -INFINITY && l < INFINITY) ? l : 0.0f;
    }
}

// Z-order key of one point from its D coordinates (B = 16 / D bits per
// feature, B = 1 for D > 8): feature f's bin q_f contributes bit i at
// position i * D + f.
// Bits of q (B of them) moved to every D-th position, bit i to i * D.
template <int D>
__device__ __forceinline__ uint32_t spread_bits(uint32_t q) {
    if constexpr (D == 4) {  // 4 bits -> 0, 4, 8, 12
        q = (q | (q << 6)) & 0x0303u;
        return (q | (q << 3)) & 0x1111u;
    } else if constexpr (D == 2) {  // 8 bits -> 0, 2, ..., 14
        q = (q | (q << 4)) & 0x0f0fu;
        q = (q | (q << 2)) & 0x3333u;
        return (q | (q << 1)) & 0x5555u;
    } else if constexpr (D == 8) {  // 2 bits -> 0, 8
        return (q & 1u) | ((q & 2u) << 7);
    } else {
        constexpr uint32_t B = D >= 16 ? 1u : 16u / D;
        uint32_t r = 0;
#pragma unroll
        for (uint32_t i = 0; i < B; ++i) r |= ((q >> i) & 1u) << (i * D);
        return r;
    }
}

template <int D>
__device__ __forceinline__ uint32_t z_key(const float (&v)[D], const float* s_lo, const float* s_scale) {
    constexpr uint32_t B = D >= 16 ? 1u : 16u / D;
    constexpr float TOP = (float)((1u << B) - 1u);
    uint32_t key = 0;
#pragma unroll
    for (int f = 0; f < D; ++f) {
        // NaN and values below the range go to bin 0, above it to the top bin
        const float x = fminf(fmaxf((v[f] - s_lo[f]) * s_scale[f], 0.0f), TOP);
        key |= spread_bits<D>((uint32_t)x) << f;
    }
    return key;
}

// Chunk histograms are counted in per-warp shared tables with plain integer
// atomics (exact and order-independent), then summed per digit: warps never
// contend with each other, and lanes of one warp that meet on a digit are
// serialised by the atomic unit itself.
template <int BT>
struct WarpHist {
    uint32_t h[BT / 32][RADIX];
};

template <int BT>
__device__ __forceinline__ void hist_clear(WarpHist<BT>& wh) {
    for (uint32_t i = threadIdx.x; i < (BT / 32) * RADIX; i += BT) (&wh.h[0][0])[i] = 0u;
}

// counts[chunk][digit] = the sum of the warps' tables (after a barrier).
template <int BT>
__device__ __forceinline__ void hist_store(const WarpHist<BT>& wh, uint32_t* __restrict__ counts) {
    for (uint32_t j = threadIdx.x; j < RADIX; j += BT) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < BT / 32; ++w) t += wh.h[w][j];
        counts[(uint64_t)blockIdx.x * RADIX + j] = t;
    }
}

// keys[c0 + j] for the chunk's points (0 for the padding past n) and the
// chunk's histogram of the low key byte, counts[chunk][digit].  Every
// coordinate of the thread's IPT points is loaded before any key is formed,
// so the loads are in flight together; with 16-byte aligned rows (vec) a
// thread's points are consecutive and each feature row is read in 16-byte
// loads.
template <int D, uint32_t CH, int BT>
__global__ void __launch_bounds__(BT) key_kernel(const float* __restrict__ P, uint64_t n,
                                                 const uint32_t* __restrict__ lo_w, const uint32_t* __restrict__ hi_w,
                                                 int vec, uint16_t* __restrict__ keys, uint32_t* __restrict__ counts) {
    constexpr uint32_t IPT = CH / BT;
    static_assert(IPT % 4 == 0 || IPT == 2, "4-point groups per thread");
    constexpr uint32_t B = D >= 16 ? 1u : 16u / D;
    __shared__ WarpHist<BT> s_wh;
    __shared__ float s_lo[16], s_scale[16];
    load_range(lo_w, hi_w, D, B, s_lo, s_scale);
    hist_clear(s_wh);
    uint32_t* my_hist = s_wh.h[threadIdx.x >> 5];
    const uint64_t c0 = (uint64_t)blockIdx.x * CH;
    const bool seq = vec && IPT % 4 == 0;  // thread's points consecutive
    float v[IPT][D];
    if (seq && c0 + CH <= n) {
        const uint64_t p0 = c0 + (uint64_t)IPT * threadIdx.x;
#pragma unroll
        for (int f = 0; f < D; ++f)
#pragma unroll
            for (uint32_t r = 0; r < IPT; r += 4) {
                const float4 q = __ldg(reinterpret_cast<const float4*>(P + (size_t)f * n + p0 + r));
                v[r][f] = q.x;
                v[r + 1][f] = q.y;
                v[r + 2][f] = q.z;
                v[r + 3][f] = q.w;
            }
    } else {
#pragma unroll
        for (uint32_t r = 0; r < IPT; ++r) {
            const uint64_t p = seq ? c0 + (uint64_t)IPT * threadIdx.x + r : c0 + r * BT + threadIdx.x;
#pragma unroll
            for (int f = 0; f < D; ++f) v[r][f] = p < n ? __ldg(P + (size_t)f * n + p) : 0.0f;
        }
    }
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < IPT; ++r) {
        const uint64_t p = seq ? c0 + (uint64_t)IPT * threadIdx.x + r : c0 + r * BT + threadIdx.x;
        const uint32_t key = p < n ? z_key<D>(v[r], s_lo, s_scale) : 0u;
        keys[p] = (uint16_t)key;
        if (p < n) atomicAdd(&my_hist[key & (RADIX - 1u)], 1u);
    }
    __syncthreads();
    hist_store(s_wh, counts);
}

template <int D>
void launch_key_kernel(uint64_t chunks, const float* P, uint64_t n, const uint32_t* lo, const uint32_t* hi, int vec,
                       uint16_t* keys, uint32_t* counts, cudaStream_t s) {
    key_kernel<D, chunk_of(D), SB><<<(unsigned)chunks, SB, 0, s>>>(P, n, lo, hi, vec, keys, counts);
}

void launch_keys(uint32_t d, uint64_t chunks, const float* P, uint64_t n, const uint32_t* lo, const uint32_t* hi,
                 int vec, uint16_t* keys, uint32_t* counts, cudaStream_t s) {
    switch (d) {
#define CKM_KEY_CASE(DD) \
    case DD: launch_key_kernel<DD>(chunks, P, n, lo, hi, vec, keys, counts, s); break;
        CKM_KEY_CASE(1) CKM_KEY_CASE(2) CKM_KEY_CASE(3) CKM_KEY_CASE(4) CKM_KEY_CASE(5) CKM_KEY_CASE(6)
        CKM_KEY_CASE(7) CKM_KEY_CASE(8) CKM_KEY_CASE(9) CKM_KEY_CASE(10) CKM_KEY_CASE(11) CKM_KEY_CASE(12)
        CKM_KEY_CASE(13) CKM_KEY_CASE(14) CKM_KEY_CASE(15)
#undef CKM_KEY_CASE
        default: launch_key_kernel<16>(chunks, P, n, lo, hi, vec, keys, counts, s); break;
    }
}

// counts[chunk][digit] of the key byte at `shift` over a padded key array.
template <uint32_t CH, int BT>
__global__ void __launch_bounds__(BT) hist_kernel(const uint16_t* __restrict__ keys, uint64_t n, uint32_t shift,
                                                  uint32_t* __restrict__ counts) {
    constexpr uint32_t IPT = CH / BT;  // 8, 4 or 2 consecutive keys per thread: one 16, 8 or 4-byte load
    __shared__ WarpHist<BT> s_wh;
    hist_clear(s_wh);
    __syncthreads();
    uint32_t* my_hist = s_wh.h[threadIdx.x >> 5];
    const uint64_t p0 = (uint64_t)blockIdx.x * CH + threadIdx.x * IPT;
    uint16_t k[IPT];
    if constexpr (IPT == 8) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(keys + p0));
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            k[2 * i] = (uint16_t)(w[i] & 0xffffu);
            k[2 * i + 1] = (uint16_t)(w[i] >> 16);
        }
    } else if constexpr (IPT == 4) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(keys + p0));
        k[0] = (uint16_t)(v.x & 0xffffu);
        k[1] = (uint16_t)(v.x >> 16);
        k[2] = (uint16_t)(v.y & 0xffffu);
        k[3] = (uint16_t)(v.y >> 16);
    } else {
        static_assert(IPT == 2, "2, 4 or 8 keys per thread");
        const uint32_t v = __ldg(reinterpret_cast<const unsigned int*>(keys + p0));
        k[0] = (uint16_t)(v & 0xffffu);
        k[1] = (uint16_t)(v >> 16);
    }
#pragma unroll
    for (uint32_t r = 0; r < IPT; ++r)
        if (p0 + r < n) atomicAdd(&my_hist[((uint32_t)k[r] >> shift) & (RADIX - 1u)], 1u);
    __syncthreads();
    hist_store(s_wh, counts);
}

// --- exclusive scan of counts[chunk][digit] in digit-major order ----------
// partial[blk][digit] = the total of the digit over the block's SCAN_ROWS chunks
__global__ void __launch_bounds__(RADIX) scan_partial_kernel(const uint32_t* __restrict__ counts, uint64_t rows,
                                                             uint32_t* __restrict__ partial) {
    const uint64_t r0 = (uint64_t)blockIdx.x * SCAN_ROWS;
    const uint64_t r1 = min(rows, r0 + SCAN_ROWS);
    uint32_t t = 0;
    for (uint64_t r = r0; r < r1; r += SCAN_BATCH) {
        uint32_t v[SCAN_BATCH];
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i) v[i] = r + i < r1 ? counts[(r + i) * RADIX + threadIdx.x] : 0u;
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i) t += v[i];
    }
    partial[(uint64_t)blockIdx.x * RADIX + threadIdx.x] = t;
}

// One CTA: partial[blk][digit] becomes the exclusive prefix of the digit
// over the blocks, and row nblk the start of each digit's output range (the
// totals of the smaller digits).
__global__ void __launch_bounds__(RADIX) scan_top_kernel(uint32_t* __restrict__ partial, uint32_t nblk) {
    __shared__ uint32_t s_w[RADIX / 32];
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    uint32_t run = 0;
    for (uint32_t b0 = 0; b0 < nblk; b0 += SCAN_BATCH) {
        uint32_t v[SCAN_BATCH];
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i) v[i] = b0 + i < nblk ? partial[(uint64_t)(b0 + i) * RADIX + t] : 0u;
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i)
            if (b0 + i < nblk) {
                partial[(uint64_t)(b0 + i) * RADIX + t] = run;
                run += v[i];
            }
    }
    uint32_t incl = run;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    uint32_t base = incl - run;
    for (uint32_t w = 0; w < warp; ++w) base += s_w[w];
    partial[(uint64_t)nblk * RADIX + t] = base;
}

// counts[chunk][digit] = where the chunk's run of the digit starts
__global__ void __launch_bounds__(RADIX) scan_apply_kernel(uint32_t* __restrict__ counts, uint64_t rows,
                                                           const uint32_t* __restrict__ partial, uint32_t nblk) {
    const uint64_t r0 = (uint64_t)blockIdx.x * SCAN_ROWS;
    const uint64_t r1 = min(rows, r0 + SCAN_ROWS);
    uint32_t run = partial[(uint64_t)blockIdx.x * RADIX + threadIdx.x] + partial[(uint64_t)nblk * RADIX + threadIdx.x];
    for (uint64_t r = r0; r < r1; r += SCAN_BATCH) {
        uint32_t v[SCAN_BATCH];
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i) v[i] = r + i < r1 ? counts[(r + i) * RADIX + threadIdx.x] : 0u;
#pragma unroll
        for (uint32_t i = 0; i < SCAN_BATCH; ++i)
            if (r + i < r1) {
                counts[(r + i) * RADIX + threadIdx.x] = run;
                run += v[i];
            }
    }
}

// --- one scatter pass ------------------------------------------------------
// Dynamic shared memory: s_pts [d][CH] f32, s_key [CH] u16, s_src [CH] u16,
// s_idx [CH] u32 (only with idx_in).
size_t scatter_smem(uint32_t d, bool with_idx) {
    const size_t ch = chunk_items(d);
    return ch * d * 4 + ch * 2 + ch * 2 + (with_idx ? ch * 4 : 0);
}

template <uint32_t CH, int BT>
__global__ void __launch_bounds__(BT, 1024 / BT)
    scatter_kernel(const float* __restrict__ P, const uint32_t* __restrict__ idx_in, const uint16_t* __restrict__ keys,
                   uint64_t n, uint32_t d, uint32_t shift, const uint32_t* __restrict__ offsets, int vec,
                   float* __restrict__ P_out, uint16_t* __restrict__ keys_out, uint32_t* __restrict__ idx_out) {
    constexpr uint32_t NW = BT / 32;
    constexpr uint32_t IPW = CH / NW;        // items of a warp (a contiguous run)
    constexpr uint32_t ROUNDS = IPW / 32;
    extern __shared__ __align__(16) unsigned char smem[];
    float* s_pts = reinterpret_cast<float*>(smem);
    uint16_t* s_key = reinterpret_cast<uint16_t*>(s_pts + (size_t)d * CH);
    uint16_t* s_src = s_key + CH;
    uint32_t* s_idx = reinterpret_cast<uint32_t*>(s_src + CH);
    // per warp and digit: the count of the digit in the warp's earlier
    // rounds, then (after the scan) the digit's items in earlier warps
    __shared__ uint16_t s_wh[NW][RADIX];
    __shared__ uint32_t s_off[RADIX], s_base[RADIX], s_wsum[RADIX / 32];

    const uint64_t c0 = (uint64_t)blockIdx.x * CH;
    const uint32_t valid = (uint32_t)min((uint64_t)CH, n - c0);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

    // 1. stage the keys (group 0), then the points and indices (group 1)
    stage_words<BT>(reinterpret_cast<uint32_t*>(s_key), reinterpret_cast<const uint32_t*>(keys + c0), CH / 2, true);
    cp_async_commit();
    for (uint32_t f = 0; f < d; ++f)
        stage_words<BT>(reinterpret_cast<uint32_t*>(s_pts + (size_t)f * CH),
                        reinterpret_cast<const uint32_t*>(P + (size_t)f * n + c0), valid, vec != 0);
    if (idx_in) stage_words<BT>(s_idx, idx_in + c0, valid, true);
    cp_async_commit();
    for (uint32_t t = lane; t < RADIX; t += 32) s_wh[warp][t] = 0;
    cp_async_wait<1>();
    __syncthreads();

    // 2. stable ranks within (warp, digit): warp w owns items
    //    [w * IPW, (w + 1) * IPW), in rounds of 32 consecutive items
    uint32_t dig[ROUNDS], rank[ROUNDS];
#pragma unroll
    for (uint32_t r = 0; r < ROUNDS; ++r) {
        const uint32_t j = warp * IPW + r * 32 + lane;
        const bool ok = j < valid;
        const uint32_t active = __ballot_sync(0xffffffffu, ok);
        dig[r] = 0;
        rank[r] = 0;
        if (ok) {
            const uint32_t dg = ((uint32_t)s_key[j] >> shift) & (RADIX - 1u);
            const uint32_t peers = __match_any_sync(active, dg);
            dig[r] = dg;
            rank[r] = (uint32_t)s_wh[warp][dg] + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            __syncwarp(active);  // every lane has read the count before the leader moves it
            if (lane == (uint32_t)(__ffs(peers) - 1)) s_wh[warp][dg] += (uint16_t)__popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();

    // 3. thread t < RADIX = digit t: the counts of the warps before each
    //    warp, the digit's chunk-local start, and its place in the output
    if (threadIdx.x < RADIX) {
        const uint32_t t = threadIdx.x;
        uint32_t tot = 0;
        for (uint32_t w = 0; w < NW; ++w) {
            const uint32_t v = s_wh[w][t];
            s_wh[w][t] = (uint16_t)tot;
            tot += v;
        }
        uint32_t incl = tot;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_wsum[warp] = incl;
        asm volatile("bar.sync 1, %0;" ::"r"(RADIX));  // the digit threads only
        uint32_t excl = incl - tot;
        for (uint32_t w = 0; w < warp; ++w) excl += s_wsum[w];
        s_off[t] = excl;
        s_base[t] = offsets[(uint64_t)blockIdx.x * RADIX + t] - excl;  // mod 2^32: base + q < 2^32
    }
    __syncthreads();

    // 4. sorted chunk position of each item
#pragma unroll
    for (uint32_t r = 0; r < ROUNDS; ++r) {
        const uint32_t j = warp * IPW + r * 32 + lane;
        if (j < valid) s_src[s_off[dig[r]] + s_wh[warp][dig[r]] + rank[r]] = (uint16_t)j;
    }
    cp_async_wait<0>();
    __syncthreads();

    // 5. write the runs out: consecutive sorted positions are consecutive
    //    output positions within a digit's run
    for (uint32_t q = threadIdx.x; q < valid; q += BT) {
        const uint32_t src = s_src[q];
        const uint32_t key = s_key[src];
        const uint32_t g = s_base[(key >> shift) & (RADIX - 1u)] + q;
        for (uint32_t f = 0; f < d; ++f) P_out[(size_t)f * n + g] = s_pts[(size_t)f * CH + src];
        if (keys_out) keys_out[g] = (uint16_t)key;
        if (idx_out) idx_out[g] = idx_in ? s_idx[src] : (uint32_t)(c0 + src);
    }
}

__global__ void __launch_bounds__(256) unpermute_kernel(uint64_t n, const uint32_t* __restrict__ perm,
                                                        const uint32_t* __restrict__ in, uint32_t* __restrict__ out) {
    for (uint64_t q = (uint64_t)blockIdx.x * 256 + threadIdx.x; q < n; q += (uint64_t)gridDim.x * 256)
        out[perm[q]] = in[q];
}

uint32_t grid_of(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    const uint64_t cap = (uint64_t)device_info().sm_count * 8;
    if (g > cap) g = cap;
    return (uint32_t)(g < 1 ? 1 : g);
}

int scan_offsets(uint32_t* counts, uint32_t* partial, uint64_t chunks, cudaStream_t s) {
    const uint64_t nblk = scan_blocks_of(chunks);
    scan_partial_kernel<<<(unsigned)nblk, RADIX, 0, s>>>(counts, chunks, partial);
    scan_top_kernel<<<1, RADIX, 0, s>>>(partial, (uint32_t)nblk);
    scan_apply_kernel<<<(unsigned)nblk, RADIX, 0, s>>>(counts, chunks, partial, (uint32_t)nblk);
    return 3;
}

template <uint32_t CH, int BT>
int set_scatter_smem(uint32_t d) {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return CKM_OK;
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, scatter_kernel<CH, BT>);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(spatial scatter)");
    if (fa.sharedSizeBytes + scatter_smem(d, true) > device_info().smem_optin)
        return fail(CKM_ERR_UNSUPPORTED, "spatial sort: the scatter's staging buffers exceed shared memory");
    e = cudaFuncSetAttribute(scatter_kernel<CH, BT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(device_info().smem_optin - fa.sharedSizeBytes));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(spatial scatter)");
    if (dev >= 0 && dev < 64) done[dev] = true;
    return CKM_OK;
}

template <uint32_t CH, int BT>
int sort_passes(uint32_t d, uint64_t n, const float* points, float* sorted, uint32_t* perm, const SortWs& ws,
                cudaStream_t s) {
    int st = set_scatter_smem<CH, BT>(d);
    if (st != CKM_OK) return st;
    const uint64_t chunks = num_chunks(n, d);
    // 16-byte copies and loads need 16-byte aligned rows: the base and n * 4
    const int vec_in = ((reinterpret_cast<uintptr_t>(points) & 15u) == 0 && (n & 3u) == 0) ? 1 : 0;
    const int vec_tmp = ((reinterpret_cast<uintptr_t>(ws.tmp_points) & 15u) == 0 && (n & 3u) == 0) ? 1 : 0;
    uint64_t launches = 0;

    const uint32_t samples = (uint32_t)std::min<uint64_t>(n, BBOX_SAMPLES);
    const uint64_t stride = n / samples;
    const unsigned bbox_grid = (unsigned)std::min<uint64_t>(256, (samples + 255) / 256);
    bbox_sample_kernel<<<bbox_grid, 256, 0, s>>>(points, n, d, stride, samples, ws.lo, ws.hi);
    launch_keys(d, chunks, points, n, ws.lo, ws.hi, vec_in, ws.keys0, ws.counts, s);
    launches += 2 + scan_offsets(ws.counts, ws.partial, chunks, s);
    scatter_kernel<CH, BT><<<(unsigned)chunks, BT, scatter_smem(d, false), s>>>(
        points, nullptr, ws.keys0, n, d, 0, ws.counts, vec_in, ws.tmp_points, ws.keys1, perm ? ws.tmp_idx : nullptr);
    hist_kernel<CH, BT><<<(unsigned)chunks, BT, 0, s>>>(ws.keys1, n, 8, ws.counts);
    launches += 2 + scan_offsets(ws.counts, ws.partial, chunks, s);
    scatter_kernel<CH, BT><<<(unsigned)chunks, BT, scatter_smem(d, perm != nullptr), s>>>(
        ws.tmp_points, perm ? ws.tmp_idx : nullptr, ws.keys1, n, d, 8, ws.counts, vec_tmp, sorted, nullptr, perm);
    launches += 1;
    count_launch(launches);
    return CKM_OK;
}

}  // namespace

size_t spatial_sort_workspace_bytes(uint64_t n, uint32_t d) {
    if (d == 0) return 0;
    const WsSizes z = ws_sizes(n, d);
    return 256 + z.counts + z.partial + 2 * z.keys + z.pts + z.idx;
}

int launch_spatial_sort(uint32_t d, uint64_t n, const float* points, float* sorted, uint32_t* perm, void* ws_ptr,
                        cudaStream_t s) {
    SortWs ws = sort_ws(ws_ptr, n, d);
    // lo = all ones (min identity), hi = zero
    cudaError_t e = cudaMemsetAsync(ws.lo, 0xff, 16 * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ws.hi, 0, 16 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_fail(e, "spatial sort: workspace init");
    if (n == 0) return CKM_OK;
    const int st = d <= 4 ? sort_passes<4096, SB>(d, n, points, sorted, perm, ws, s)
                          : (d <= 8 ? sort_passes<2048, SB>(d, n, points, sorted, perm, ws, s)
                                    : sort_passes<1024, SB>(d, n, points, sorted, perm, ws, s));
    if (st != CKM_OK) return st;
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "spatial sort launch");
}

int launch_unpermute_u32(uint64_t n, const uint32_t* perm, const uint32_t* in, uint32_t* out, cudaStream_t s) {
    if (n == 0) return CKM_OK;
    unpermute_kernel<<<grid_of(n), 256, 0, s>>>(n, perm, in, out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "unpermute launch");
}

}  // namespace ckm
