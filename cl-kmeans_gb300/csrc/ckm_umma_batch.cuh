// Tensor-core (tcgen05) labelling for the batched kernel's d = 32 / 64 jobs.
//
// The 512-thread CTA works as two independent halves of 256 threads on
// alternate 128-point sub-tiles (own point tiles, own 256 TMEM columns, own
// mbarrier, own named barrier; the staged centroids are shared), so that one
// half's MMA wait and merge overlap the other half's work.  Per sub-tile a
// half splits every coordinate into two fp16 halves, x = x_h + x_l (+ a
// residual of at most 2^-22 |x_f| + 2^-25), writes both as K-major
// 128-byte-swizzled tiles, and one of its threads issues x_h.c_l and x_l.c_h,
// then x_h.c_h (tcgen05.mma kind::f16, M = 128 points, N = k_pad clusters,
// K = 16 per instruction) into one f32 accumulator in tensor memory.  The
// centroids' halves are staged the same way once per segment.  Each warp then
// reads the scores of its 32 points (its TMEM lane quarter) for its half of
// the clusters, s_c = |c|^2 - 2 dot, keeps the lowest two, and the
// certificate below decides the label.  Points it does not prove are
// deferred: their candidates (the clusters within T of the lowest score) are
// resolved later with the reference's arithmetic; points whose values are not
// finite take the full exact scan at once.  The point sums use the FP32
// coordinates held in registers.
//
// Certificate.  With a >= |x|, cm >= max_c |c|, r = a + cm, eps = 2^-25 sqrt(D)
// and gamma = 2 D 2^-23 (f32 accumulation, two ulps per addition of the
// running absolute sum: the 2D cross products are issued first, so their
// partial sums stay below 2^-10 |x||c| and only the D products x_h c_h add
// errors of the full size):
//   |dot - x.c| <= 3.001 2^-22 a cm + 1.01 eps (a + cm) + gamma 1.01 (a + eps)(cm + eps)
// (the dropped x_l.c_l term and the two residuals), the score adds the
// roundings of |c|^2 and of fma(-2, dot, |c|^2), and the reference's FP32
// distance is within (D + 4) 2^-24 of the exact one.  So
//   T = A_D r^2 + B_D r + C_D,
//   A_D = (3.001 2^-22 + 1.01 gamma + 5.2 2^-24 + 2 (D + 4) 2^-24) 1.001,
//   B_D = 4.1 eps,  C_D = 2^-40 (second-order and underflow terms),
// and m2 - m1 > T proves that the cluster of m1 is strictly nearest in the
// reference's arithmetic.  The proof needs finite values below fp16's range:
// a < 2^15 per point, cm < 2^15 per segment (checked when staging), r^2 < 2^120.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ckm_batched.h"
#include "ckm_device.cuh"
#include "ckm_mma_screen.cuh"
#include "ckm_umma.cuh"

namespace ckm {

constexpr uint32_t UMMA_M = 128;             // points per sub-tile (TMEM lanes)
constexpr uint32_t UMMA_HALF_COLS = 256;     // accumulator columns of one half (>= UMMA_MAX_K)
constexpr uint32_t UMMA_TMEM_COLS = 2 * UMMA_HALF_COLS;
constexpr float UMMA_MAX_ABS = 32768.0f;     // |x| and max |c| below this: no fp16 overflow
constexpr unsigned long long UMMA_WAIT_NS = 2000000000ull;
constexpr uint32_t UMMA_TILE_BYTES = UMMA_M * 128u;  // one operand tile of 128 rows

// Clusters padded to a multiple of 32 (two column groups of whole 16-column
// loads per half; padded clusters have |c|^2 = +inf and never win).
__host__ __device__ __forceinline__ uint32_t umma_k_pad(uint32_t k) { return (k + 31u) & ~31u; }

// Operand tiles of a tensor-core segment in dynamic shared memory, from a
// 1024-byte aligned base: centroid halves (k_pad rows each), then per CTA
// half its point halves (128 rows each); rows of 128 bytes.
struct UmmaLayout {
    uint32_t bh, bl, a, end;
};

__host__ __device__ __forceinline__ UmmaLayout umma_layout(uint32_t kp) {
    UmmaLayout L;
    L.bh = 0;
    L.bl = kp * 128u;
    L.a = 2u * kp * 128u;  // half h: hi at a + 2 h TILE, lo at a + (2 h + 1) TILE
    L.end = L.a + 4u * UMMA_TILE_BYTES;
    return L;
}

// Bytes a tensor-core segment needs in front of its sum table (with the
// alignment slack of the dynamic shared-memory base).
__host__ __device__ __forceinline__ size_t umma_region_bytes(uint32_t k) {
    return 1024u + umma_layout(umma_k_pad(k)).end;
}

// Unproved points with finite values are deferred: the scan of their scores
// records (point, candidate) pairs, and all threads resolve the pairs together
// at the end of the tile range (one exact distance per thread; the
// lexicographic (distance, index) minimum per point through a 64-bit
// atomicMin), so no warp stalls its half on the latency of an exact distance.
// A point the list has no room for is resolved on the spot.
constexpr uint32_t UMMA_CHUNK = 16384;    // points between resolutions
constexpr uint32_t UMMA_DEF_CAP = 384;    // deferred points per chunk
constexpr uint32_t UMMA_PAIR_CAP = 1536;  // their candidate pairs (deferred index << 16 | cluster)

// Per-sub-tile scratch of the two halves, a static shared-memory object so
// that its addresses cost no registers.  [half][group][point] and [half][point].
struct __align__(16) UmmaScratch {
    unsigned long long def_key[UMMA_DEF_CAP];  // (distance bits << 32 | cluster), minimum
    float cn[UMMA_MAX_K];            // |c|^2 (+inf for padding); read as float4
    float m1[4 * UMMA_M], m2[4 * UMMA_M], nx[4 * UMMA_M];
    uint32_t i1[4 * UMMA_M];
    uint32_t lab[2 * UMMA_M], mode[2 * UMMA_M], didx[2 * UMMA_M];
    float cut[2 * UMMA_M];
    uint32_t def_p[UMMA_DEF_CAP];    // point offset from the start of the chunk
    uint32_t pair[UMMA_PAIR_CAP];
    unsigned int ndef, npair, need[2];
    unsigned int abort[2];           // per half: its wait for the tensor cores ran out
};

namespace umma_detail {

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool try_wait_hint(uint32_t bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

// Waits for the phase with a time limit; false when it did not complete.
// One thread waits (the others are at a barrier), so it polls without a
// suspend hint first: the MMAs of a sub-tile take about a microsecond.
__device__ __forceinline__ bool wait_bounded(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    for (int i = 0; i < 4096; ++i)
        if (umma::mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (;;) {
        if (try_wait_hint(bar, parity, 20000u)) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

// Barrier of one 256-thread half (ids 1 and 2; 0 is __syncthreads).
__device__ __forceinline__ void half_sync(uint32_t half) {
    asm volatile("bar.sync %0, 256;" ::"r"(1u + half) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// x = hi + lo (+ residual): hi = fp16(x), lo = fp16(x - hi); x - hi is exact
// in FP32.  Two values per 32-bit word, the lower feature in the low half.
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __half2 h = __floats2half2_rn(a, b);  // one packed conversion (a in the low half)
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Eight consecutive features of row r as hi and lo chunks of the two tiles.
__device__ __forceinline__ void store_chunk(uint32_t hi_base, uint32_t lo_base, uint32_t r, uint32_t f0,
                                            const float* v) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) split2(v[2 * e], v[2 * e + 1], h[e], l[e]);
    const uint32_t off = umma::sw128_offset(r, f0);
    st_shared_v4(hi_base + off, h[0], h[1], h[2], h[3]);
    st_shared_v4(lo_base + off, l[0], l[1], l[2], l[3]);
}

// Instruction descriptor, kind::f16 with fp16 A and B (format 0), f32 D,
// both operands K-major.
__device__ __forceinline__ uint32_t idesc_f16(uint32_t M, uint32_t N) {
    return (1u << 4) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// The reference distance (kmeans_naive.cpp:52-57) of point p to cluster c:
// t = x_f - c_f, acc = fma(t, t, acc), f ascending; column-major operands.
template <int D>
__device__ __forceinline__ float exact_distance_cm(const float* __restrict__ P, uint64_t n, uint64_t p,
                                                   const float* __restrict__ C, uint32_t k, uint32_t c) {
    float acc = 0.0f;
#pragma unroll 16
    for (int f = 0; f < D; ++f) {
        const float t = __ldg(P + (size_t)f * n + p) - __ldg(C + (size_t)f * k + c);
        acc = f == 0 ? t * t : fmaf(t, t, acc);
    }
    return acc;
}

template <int D>
struct UmmaBound {
    static constexpr float gamma = 2.0f * (float)D * 0x1p-23f * 1.005f;
    static constexpr float A =
        (3.001f * 0x1p-22f + 1.01f * gamma + 5.2f * 0x1p-24f + 2.0f * (float)(D + 4) * 0x1p-24f) * 1.001f;
    static constexpr float B = 4.1f * 0x1p-25f * (D == 64 ? 8.0f : 6.0f) * 1.001f;
    static constexpr float C = 0x1p-40f;
};

}  // namespace umma_detail

// Stages the segment's centroids: fp16 hi / lo rows (K-major, swizzled),
// |c|^2 (FP64 sum rounded once; NaN for a NaN centroid, +inf for padding) and
// max |c| over the non-NaN centroids (rounded up) into *cm_bits.
template <int D, int BT>
__device__ __forceinline__ void umma_stage(const float* __restrict__ C, uint32_t k, uint32_t base,
                                           const UmmaLayout& L, uint32_t kp, float* s_cn, unsigned int* cm_bits) {
    constexpr uint32_t CH = D / 8;
    for (uint32_t i = threadIdx.x; i < kp * CH; i += BT) {
        const uint32_t c = i % kp, j = i / kp;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = c < k ? __ldg(C + (size_t)(8 * j + e) * k + c) : 0.0f;
        umma_detail::store_chunk(base + L.bh, base + L.bl, c, 8 * j, v);
    }
    for (uint32_t c = threadIdx.x; c < kp; c += BT) {
        if (c < k) {
            double s = 0.0;
#pragma unroll 8
            for (int f = 0; f < D; ++f) {
                const double v = (double)__ldg(C + (size_t)f * k + c);
                s = fma(v, v, s);
            }
            s_cn[c] = (float)s;
            if (!isnan(s)) atomicMax(cm_bits, __float_as_uint(__double2float_ru(sqrt(s) * (1.0 + 0x1p-40))));
        } else {
            s_cn[c] = __int_as_float(0x7f800000);
        }
    }
}

// Resolves the deferred points (every thread calls it): exact distances of
// the candidate pairs, then per point the label, its mass and its sums.
template <int D, int BT>
__device__ __forceinline__ void umma_resolve(const BatchJobDev& J, const float* __restrict__ C, uint64_t begin,
                                             UmmaScratch& us, float* s_sum, unsigned int* s_mass, uint32_t copies) {
    __syncthreads();  // the lists are complete
    const uint64_t n = J.n;
    const uint32_t k = J.k;
    const float* __restrict__ P = J.points;
    const uint32_t np = min(us.npair, UMMA_PAIR_CAP), nd = min(us.ndef, UMMA_DEF_CAP);
    for (uint32_t i = threadIdx.x; i < np; i += BT) {
        const uint32_t d = us.pair[i] >> 16, c = us.pair[i] & 0xffffu;
        const float dist = umma_detail::exact_distance_cm<D>(P, n, begin + us.def_p[d], C, k, c);
        if (dist < FLT_MAX)
            atomicMin(&us.def_key[d], ((unsigned long long)__float_as_uint(dist) << 32) | (unsigned long long)c);
    }
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    for (uint32_t d = warp; d < nd; d += BT / 32) {
        const uint64_t p = begin + us.def_p[d];
        const unsigned long long key = us.def_key[d];
        const uint32_t lab = key == ~0ull ? 0u : (uint32_t)key;  // nothing below FLT_MAX: cluster 0
        if (lane == 0) {
            J.labels[p] = lab;
            if (copies) atomicAdd(&s_mass[lab], 1u);
            else atomicAdd(&J.msum[lab], 1ull);
        }
        for (uint32_t f = lane; f < (uint32_t)D; f += 32) {
            const float v = __ldg(P + (size_t)f * n + p);
            if (copies) atomicAdd(&s_sum[((size_t)f * k + lab) * copies + (lane & (copies - 1u))], v);
            else atomicAdd(&J.sums[(size_t)f * k + lab], (double)v);
        }
    }
    __syncthreads();
}

// Labels the points of tiles [t0, t1) of one job on the tensor cores and adds
// them into the shared table (512 threads; two halves on alternate
// sub-tiles).  bars: the halves' mbarriers (8 bytes apart); phase: this
// thread's half's next phase.  test_stall: the failure-detection test (the
// first half issues no MMA and its 1 ms wait runs out).  Returns false when a
// wait for the tensor cores ran out (every thread gets the same answer); the
// caller then stops.
template <int D>
__device__ __forceinline__ bool run_tiles_umma(const BatchJobDev& J, const float* __restrict__ C, uint32_t t0,
                                               uint32_t t1, uint32_t tile, uint32_t base, const UmmaLayout& L,
                                               uint32_t kp, uint32_t tmem, uint32_t bars, uint32_t& phase, float cm,
                                               float* s_sum, unsigned int* s_mass, uint32_t copies, UmmaScratch& us,
                                               volatile unsigned int* s_abort, bool test_stall) {
    constexpr uint32_t G = 2;            // column groups per half
    constexpr int FPT = D / (int)G;      // features per thread
    static_assert(FPT % 8 == 0, "whole 16-byte chunks per thread");
    const uint64_t n = J.n;
    const uint32_t k = J.k;
    const float* __restrict__ P = J.points;
    const uint64_t begin = (uint64_t)t0 * tile;
    const uint64_t end = min((uint64_t)t1 * tile, n);
    const uint32_t half = threadIdx.x >> 8, th = threadIdx.x & 255u;
    const uint32_t pl = th & (UMMA_M - 1u), fg = th / UMMA_M;
    const uint32_t f0 = fg * FPT;
    const uint32_t wh = th >> 5, lane = th & 31u;
    const uint32_t q = wh & 3u, h = wh >> 2;  // TMEM lane quarter (= global warp % 4), column group
    const uint32_t cpg = kp / G, c0 = h * cpg;
    const uint32_t pw = q * 32u + lane;       // the point this thread scores
    const uint32_t sA = base + L.a + half * 2u * UMMA_TILE_BYTES, sAl = sA + UMMA_TILE_BYTES;
    const uint32_t bar = bars + half * 8u;
    const uint32_t tm = tmem + half * UMMA_HALF_COLS;
    const uint32_t taddr = tm + ((q * 32u) << 16) + c0;
    const uint32_t idesc = umma_detail::idesc_f16(UMMA_M, kp);
    // scratch of this half
    float* s_m1 = us.m1 + half * G * UMMA_M;
    float* s_m2 = us.m2 + half * G * UMMA_M;
    uint32_t* s_i1 = us.i1 + half * G * UMMA_M;
    float* s_nx = us.nx + half * G * UMMA_M;
    uint32_t* s_lab = us.lab + half * UMMA_M;
    uint32_t* s_mode = us.mode + half * UMMA_M;
    uint32_t* s_didx = us.didx + half * UMMA_M;
    float* s_cut = us.cut + half * UMMA_M;
    volatile unsigned int* s_need = us.need + half;
    volatile unsigned int* my_abort = us.abort + half;
    const unsigned long long wait_ns = test_stall ? 1000000ull : UMMA_WAIT_NS;
    const float* s_cn = us.cn;
    const float INF = __int_as_float(0x7f800000);

    if (threadIdx.x == 0) {
        us.abort[0] = 0u;
        us.abort[1] = 0u;
    }
    // chunks of UMMA_CHUNK points; the deferred points of a chunk are resolved
    // at its end (both halves)
#pragma unroll 1
    for (uint64_t cb = begin; cb < end; cb += UMMA_CHUNK) {
        const uint64_t ce = min(cb + UMMA_CHUNK, end);
        if (threadIdx.x == 0) {
            us.ndef = 0u;
            us.npair = 0u;
        }
        __syncthreads();
        // d = 32: the half's next sub-tile is loaded while this one is scored (for
        // d = 64 the 32 more registers would spill; the other half overlaps the load)
        constexpr bool PREF = FPT <= 16;
        float xn[FPT];
        auto load = [&](uint64_t bb) {
            const uint64_t p = bb + pl;
#pragma unroll
            for (int i = 0; i < FPT; ++i) xn[i] = p < ce ? __ldg(P + (size_t)(f0 + i) * n + p) : 0.0f;
        };
        if (PREF && cb + half * UMMA_M < ce) load(cb + half * UMMA_M);
#pragma unroll 1
        for (uint64_t b = cb + half * UMMA_M; b < ce; b += 2 * UMMA_M) {
            // the sub-tile's points: FP32 in registers (for the sums), fp16
            // halves into this half's operand tiles
            const uint64_t end_ = ce;  // points of this chunk
            if (!PREF) load(b);
            float x[FPT];
            float nx = 0.0f;
#pragma unroll
            for (int i = 0; i < FPT; ++i) {
                x[i] = xn[i];
                nx = fmaf(x[i], x[i], nx);
            }
#pragma unroll
            for (int j = 0; j < FPT / 8; ++j) umma_detail::store_chunk(sA, sAl, pl, f0 + 8 * j, &x[8 * j]);
            s_nx[fg * UMMA_M + pl] = nx;
            umma::fence_proxy_async_smem();
            umma_detail::half_sync(half);
            if (PREF && b + 2 * UMMA_M < ce) load(b + 2 * UMMA_M);  // in flight during the MMA and the epilogue
        if (!PREF && b + 2 * UMMA_M < ce) {
            // d = 64: the next sub-tile's rows into L2 (feature th / 4, 32
            // points from 32 (th % 4)), so its loads do not wait for HBM
            const uint64_t pn = b + 2 * UMMA_M + (th & 3u) * 32u;
            if (pn < ce)
                asm volatile("prefetch.L2 [%0];" ::"l"(P + (size_t)(th >> 2) * n + pn) : "memory");
        }
            if (th == 0) {
                *s_need = 0u;
                umma::fence_after_sync();
                // failure-detection test (test_stall): the first half issues
                // no MMA, so its wait below finds nothing and runs out (1 ms)
                if (!(test_stall && half == 0)) {
                    // the small cross products first, then x_h c_h (see the bound)
#pragma unroll
                    for (uint32_t ks = 0; ks < (uint32_t)D / 16u; ++ks) {
                        const uint64_t ah = umma::sw128_desc(sA + ks * 32u);
                        const uint64_t al = umma::sw128_desc(sAl + ks * 32u);
                        const uint64_t bh = umma::sw128_desc(base + L.bh + ks * 32u);
                        const uint64_t bl = umma::sw128_desc(base + L.bl + ks * 32u);
                        umma::mma_bf16(tm, ah, bl, idesc, ks > 0 ? 1u : 0u);
                        umma::mma_bf16(tm, al, bh, idesc, 1u);
                    }
#pragma unroll
                    for (uint32_t ks = 0; ks < (uint32_t)D / 16u; ++ks)
                        umma::mma_bf16(tm, umma::sw128_desc(sA + ks * 32u),
                                       umma::sw128_desc(base + L.bh + ks * 32u), idesc, 1u);
                    umma::mma_commit(bar);
                }
                if (!umma_detail::wait_bounded(bar, phase, wait_ns)) *my_abort = 1u;
            }
            phase ^= 1u;
            umma_detail::half_sync(half);
            if (*my_abort) break;  // same value in the whole half (set before its barrier)
            umma::fence_after_sync();

            // pass 1: lowest two scores of this thread's point over its columns
            float m1 = INF, m2 = INF;
            uint32_t i1 = 0;
#pragma unroll 1
            for (uint32_t cc = 0; cc < cpg; cc += 16) {
                float v[16];
                umma::tmem_ld16(taddr + cc, v);
                const float4* cn4 = reinterpret_cast<const float4*>(s_cn + c0 + cc);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float4 cn = cn4[i];
                    const uint32_t c = c0 + cc + 4 * i;
                    screen_track(fmaf(-2.0f, v[4 * i], cn.x), c, m1, m2, i1);
                    screen_track(fmaf(-2.0f, v[4 * i + 1], cn.y), c + 1, m1, m2, i1);
                    screen_track(fmaf(-2.0f, v[4 * i + 2], cn.z), c + 2, m1, m2, i1);
                    screen_track(fmaf(-2.0f, v[4 * i + 3], cn.w), c + 3, m1, m2, i1);
                }
            }
            s_m1[h * UMMA_M + pw] = m1;
            s_m2[h * UMMA_M + pw] = m2;
            s_i1[h * UMMA_M + pw] = i1;
            umma::fence_before_sync();
            umma_detail::half_sync(half);

            // merge and certificate (one thread per point)
            if (th < UMMA_M) {
                const uint32_t p = th;
                float a1 = s_m1[p], a2 = s_m2[p];
                uint32_t ai = s_i1[p];
                screen_merge(a1, a2, ai, s_m1[UMMA_M + p], s_m2[UMMA_M + p], s_i1[UMMA_M + p]);
                const float xx = s_nx[p] + s_nx[UMMA_M + p];
                const float a = sqrtf(xx) * (1.0f + 0x1p-16f);
                const float r = (a + cm) * (1.0f + 0x1p-20f);
                const float T = fmaf(umma_detail::UmmaBound<D>::A * r, r,
                                     fmaf(umma_detail::UmmaBound<D>::B, r, umma_detail::UmmaBound<D>::C));
                const bool fin = (a1 < INF) && (a < UMMA_MAX_ABS) && (r * r < 0x1p120f) && (T < INF);
                const bool proved = fin && (a2 - a1 > T);
                // 0: labelled; 1: candidates resolved now (deferred list full);
                // 2: not finite, full exact scan now; 3: deferred
                uint32_t mode = (b + p >= end_ || proved) ? 0u : (fin ? 1u : 2u);
                if (mode == 1u) {
                    const uint32_t di = atomicAdd(&us.ndef, 1u);
                    if (di < UMMA_DEF_CAP) {
                        mode = 3u;
                        us.def_p[di] = (uint32_t)(b - cb + p);
                        us.def_key[di] = ~0ull;
                        s_didx[p] = di;
                    }
                }
                s_lab[p] = ai;
                s_cut[p] = a1 + T;
                s_mode[p] = mode;
                if (mode) *s_need = 1u;
            }
            umma_detail::half_sync(half);

            if (*s_need) {
                // pass 2 over the scores: candidates (score <= m1 + T) of deferred
                // points become pairs; modes 1 and 2 get their exact distances
                // here (candidates; every cluster), lexicographic minimum
                const uint32_t md = s_mode[pw];
                const float cut = s_cut[pw];
                const uint32_t di = md == 3u ? s_didx[pw] : 0u;
                float bd = INF;
                uint32_t bc = 0xffffffffu;
                if (__any_sync(0xffffffffu, md != 0u)) {
#pragma unroll 1
                    for (uint32_t cc = 0; cc < cpg; cc += 16) {
                        float v[16];
                        umma::tmem_ld16(taddr + cc, v);
                        if (md) {
#pragma unroll
                            for (int i = 0; i < 16; ++i) {
                                const uint32_t c = c0 + cc + i;
                                const float s = fmaf(-2.0f, v[i], s_cn[c]);
                                if (c < k && (md == 2u || s <= cut)) {
                                    if (md == 3u) {
                                        const uint32_t pi = atomicAdd(&us.npair, 1u);
                                        if (pi < UMMA_PAIR_CAP) {
                                            us.pair[pi] = (di << 16) | c;
                                            continue;
                                        }
                                    }
                                    const float dist = umma_detail::exact_distance_cm<D>(P, n, b + pw, C, k, c);
                                    if (md == 3u) {  // pair list full: straight into the point's minimum
                                        if (dist < FLT_MAX)
                                            atomicMin(&us.def_key[di], ((unsigned long long)__float_as_uint(dist) << 32) |
                                                                           (unsigned long long)c);
                                    } else if (dist < FLT_MAX && (dist < bd || (dist == bd && c < bc))) {
                                        bd = dist;
                                        bc = c;
                                    }
                                }
                            }
                        }
                    }
                }
                s_m1[h * UMMA_M + pw] = bd;
                s_i1[h * UMMA_M + pw] = bc;
                umma::fence_before_sync();
                umma_detail::half_sync(half);
                if (th < UMMA_M && (s_mode[th] == 1u || s_mode[th] == 2u)) {
                    float d1 = s_m1[th];
                    uint32_t c1 = s_i1[th];
                    const float od = s_m1[UMMA_M + th];
                    const uint32_t oc = s_i1[UMMA_M + th];
                    if (od < d1 || (od == d1 && oc < c1)) {
                        d1 = od;
                        c1 = oc;
                    }
                    s_lab[th] = c1 == 0xffffffffu ? 0u : c1;  // nothing below FLT_MAX: cluster 0
                }
                umma_detail::half_sync(half);
            }

            // labels, masses and sums (deferred points: when resolved)
            const uint64_t pt = b + pl;
            if (pt < end_ && s_mode[pl] != 3u) {
                const uint32_t lab = s_lab[pl];
                if (fg == 0) {
                    J.labels[pt] = lab;
                    if (copies) atomicAdd(&s_mass[lab], 1u);
                    else atomicAdd(&J.msum[lab], 1ull);
                }
#pragma unroll
                for (int i = 0; i < FPT; ++i) {
                    const uint32_t f = f0 + i;
                    if (copies) atomicAdd(&s_sum[((size_t)f * k + lab) * copies + (threadIdx.x & (copies - 1u))], x[i]);
                    else atomicAdd(&J.sums[(size_t)f * k + lab], (double)x[i]);
                }
            }
        }
        // after an abort this half's last MMA may still be in flight: wait for it
        // (bounded) before the caller frees the accumulator
        if (th == 0 && *my_abort) umma_detail::wait_bounded(bar, phase ^ 1u, wait_ns);
        __syncthreads();  // both halves are done with the chunk
        if (us.abort[0] || us.abort[1]) {
            if (threadIdx.x == 0) *s_abort = 1u;
            return false;
        }
        if (us.ndef) umma_resolve<D, 512>(J, C, cb, us, s_sum, s_mass, copies);
    }
    return true;
}

}  // namespace ckm
