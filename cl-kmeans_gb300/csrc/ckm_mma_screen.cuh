// Tensor-core screen for d = 32 / 64 labels (warp-level mma.sync TF32), with
// the certified bound and an exact fallback that keep the reference's labels.
//
// One warp labels 16 points at a time.  The score s_c = |c|^2 - 2 x.c comes
// from m16n8k8 TF32 MMAs (rows = points, columns = clusters, K = features)
// in a three-term split: x = x_hi + x_mid and c = c_hi + c_mid exactly
// (x_hi = x rounded to TF32, x_mid = x - x_hi, which FP32 holds exactly), and
//   dot = x_mid.c_hi + x_hi.c_mid + x_hi.c_hi
// accumulated in FP32.  The MMA reads x_mid / c_mid as TF32 (their low 13
// bits dropped or rounded): an error of at most 2^-10 |x_mid| <= 2^-21 |x|.
//
// Bound on the score error, with r >= |x| + max|c| and u = 2^-24:
//   split:        |x_mid.c_mid| + 2^-10 (|x_mid||c_hi| + |x_hi||c_mid|)
//                 <= 5 * 2^-22 |x| |c|
//   accumulation: the three products accumulate in three chains (mid x hi,
//                 hi x mid, hi x hi), and every product term may cost 2 ulps
//                 of its chain's running sum (the convention of the tcgen05
//                 path).  A chain's running sum is at most the sum of its
//                 |terms|: D terms of the hi x hi chain sum to <= |x||c|,
//                 each mid chain's to <= 2^-11 (1.001) |x||c|, so the chains
//                 cost <= D (1 + 2^-9) 2^-22 |x||c|, plus two roundings
//                 adding them up (<= 2^-23 |x||c|)
//   score:        s = fma(-2, dot, cn): 2 * dot error + rounding of cn and of
//                 the fma, <= 2u (|c|^2 + 2|x||c|)
// so B = (D + 7) 2^-23 r^2 covers it (|x||c| <= r^2 / 4, |c|^2 + 2|x||c|
// <= r^2); with the reference's own rounding rho = (D + 4) u (see
// label_rows_screened), m2 - m1 > T = 2B + 2 rho r^2 proves the label.  T is
// taken as ((D + 8) 2^-22 + (2D + 8) 2^-24) r^2 (1.001) + 2^-117 (r + 1);
// the last term covers tensor-core inputs and partial sums flushed from the
// subnormal range (at most 2^-126 per product operand and per step).
//
// Points that the bound does not prove (ties, near ties, NaN / infinite
// values, r^2 >= 2^120) are labelled exactly by the whole warp: lanes take
// clusters c = lane, lane + 32, ..., each runs the reference's sequential
// t = x - c, fma(t, t, acc) chain over the features, and the warp takes the
// lexicographic (distance, index) minimum with the reference's start value
// FLT_MAX (no distance below it: label 0).
#pragma once

#include "ckm_device.cuh"

namespace ckm {

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Shared-memory layout of the centroids for the MMA screen (they are the A
// operand: 16 clusters x 8 features per MMA).  For m-tile mt (clusters
// 16 mt .. 16 mt + 15), k-step ks (features 8 ks .. 8 ks + 7) and lane
// (g = lane / 4, t = lane % 4) two float4, [hi] then [mid], each
//   { a(g, t), a(g + 8, t), a(g, t + 4), a(g + 8, t + 4) },
// a(r, j) = centroid 16 mt + r, feature 8 ks + j: that lane's A fragment of
// the MMA pair, read with two conflict-free 128-bit loads.  hi + mid is the
// FP32 centroid exactly.  Clusters k .. k_pad - 1 are zero, with cn = NaN.
__device__ __forceinline__ size_t mma_frag_index(uint32_t mt, uint32_t ks, uint32_t part, uint32_t lane,
                                                 uint32_t KS) {
    return (((size_t)mt * KS + ks) * 2 + part) * 32 + lane;
}

__host__ __device__ __forceinline__ uint32_t mma_k_pad(uint32_t k) { return (k + 15u) & ~15u; }

// Shared bytes of the MMA centroid fragments plus |c|^2 (16-byte multiple).
__host__ __device__ __forceinline__ size_t mma_cent_bytes(uint32_t k, uint32_t d) {
    const size_t k_pad = mma_k_pad(k);
    return ((k_pad * d * 2 + k_pad) * sizeof(float) + 15) & ~size_t(15);
}

// Smallest k that takes the tensor-core screen.  Below it the per-8-point
// overhead outweighs the MMAs and the FP32 screen is faster (one step of the
// batched mixture's d = 32 jobs with k in [16, 32) / [32, 64): 0.91 / 1.53 ms
// on the FP32 screen against 1.33 / 1.75 ms on the tensor cores; d = 64,
// k in [16, 32) / [32, 64): 2.10 / 3.15 ms against 2.36 / 2.72 ms).
__host__ __device__ __forceinline__ uint32_t mma_min_k(uint32_t d) { return d == 64 ? 32u : 64u; }

// Stages the column-major centroids C[f * k + c] into that layout and
// cn[c] = |c|^2 (FP64 sum, one rounding; NaN for padding), and the maximum of
// the non-NaN cn into *s_cn_max (zeroed by the caller).  All threads of the
// CTA; a barrier must follow.
template <int D>
__device__ __forceinline__ void mma_stage_centroids(const float* __restrict__ C, uint32_t k, float4* frag, float* cn,
                                                    unsigned int* s_cn_max, uint32_t tid, uint32_t nthreads) {
    constexpr uint32_t KS = D / 8;
    const uint32_t k_pad = mma_k_pad(k);
    const uint32_t total = (k_pad / 16) * KS * 32;
    for (uint32_t i = tid; i < total; i += nthreads) {
        const uint32_t lane = i & 31u, ks = (i >> 5) % KS, mt = (i >> 5) / KS;
        const uint32_t c0 = mt * 16 + (lane >> 2), f0 = ks * 8 + (lane & 3u);
        float v[4], h[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t c = c0 + ((j & 1) ? 8u : 0u), f = f0 + ((j & 2) ? 4u : 0u);
            v[j] = c < k ? C[(size_t)f * k + c] : 0.0f;
            h[j] = __uint_as_float(to_tf32(v[j]));
        }
        frag[mma_frag_index(mt, ks, 0, lane, KS)] = make_float4(h[0], h[1], h[2], h[3]);
        frag[mma_frag_index(mt, ks, 1, lane, KS)] = make_float4(v[0] - h[0], v[1] - h[1], v[2] - h[2], v[3] - h[3]);
    }
    for (uint32_t c = tid; c < k_pad; c += nthreads) {
        float v = __int_as_float(0x7fc00000);
        if (c < k) {
            double s = 0.0;
            for (uint32_t f = 0; f < (uint32_t)D; ++f) {
                const double e = (double)C[(size_t)f * k + c];
                s = fma(e, e, s);
            }
            v = (float)s;
            if (!isnan(v)) atomicMax(s_cn_max, __float_as_uint(v));
        }
        cn[c] = v;
    }
}

// Exact centroid element (c, f) from the fragment layout.
template <int D>
__device__ __forceinline__ float mma_centroid(const float4* frag, uint32_t c, uint32_t f) {
    const uint32_t r = c & 15u, lane = ((r & 7u) << 2) | (f & 3u), j = (r >> 3) | (((f >> 2) & 1u) << 1);
    const size_t i = mma_frag_index(c >> 4, f >> 3, 0, lane, D / 8);
    const float* hi = reinterpret_cast<const float*>(frag + i);
    const float* mid = reinterpret_cast<const float*>(frag + i + 32);
    return hi[j] + mid[j];
}

// Merges another lane's (m1, m2, i1) into this one (lowest and second lowest
// score; i1 belongs to m1).
__device__ __forceinline__ void screen_merge(float& m1, float& m2, uint32_t& i1, float om1, float om2, uint32_t oi1) {
    const bool lt = om1 < m1;
    m2 = fminf(fminf(m2, om2), lt ? m1 : om1);
    i1 = lt ? oi1 : i1;
    m1 = lt ? om1 : m1;
}

// Exact label of point p by the whole warp (all 32 lanes must call it).
template <int D>
__device__ __forceinline__ uint32_t warp_exact_label(const float* __restrict__ P, uint64_t n, uint64_t p,
                                                     const float4* frag, uint32_t k, uint32_t lane) {
    float best = FLT_MAX;
    uint32_t lab = 0xffffffffu;
#pragma unroll 1
    for (uint32_t c = lane; c < k; c += 32) {
        float acc = 0.0f;
#pragma unroll 4
        for (uint32_t f = 0; f < (uint32_t)D; ++f) {
            const float t = __ldg(P + (size_t)f * n + p) - mma_centroid<D>(frag, c, f);
            acc = f == 0 ? t * t : fmaf(t, t, acc);
        }
        if (acc < best) {
            best = acc;
            lab = c;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t ol = __shfl_xor_sync(0xffffffffu, lab, o);
        if (ob < best || (ob == best && ol < lab)) {
            best = ob;
            lab = ol;
        }
    }
    return lab == 0xffffffffu ? 0u : lab;
}

// One m-tile (16 clusters) against the warp's 8 points: mid x hi, hi x mid
// and hi x hi products accumulate in three separate chains, added at the end
// (the accumulation bound above covers any grouping of the terms).
template <int D>
__device__ __forceinline__ void mma_tile(const float4* __restrict__ frag, uint32_t mt, uint32_t lane,
                                         const uint32_t (&bh)[D / 4], const uint32_t (&bm)[D / 4], float (&acc)[4]) {
    constexpr uint32_t KS = D / 8;
    float p[4] = {0.0f, 0.0f, 0.0f, 0.0f}, q[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] = 0.0f;
#pragma unroll
    for (uint32_t ks = 0; ks < KS; ++ks) {
        const float4 h = frag[mma_frag_index(mt, ks, 0, lane, KS)];
        const float4 m = frag[mma_frag_index(mt, ks, 1, lane, KS)];
        const uint32_t h0 = __float_as_uint(h.x), h1 = __float_as_uint(h.y), h2 = __float_as_uint(h.z),
                       h3 = __float_as_uint(h.w);
        mma_tf32(p, __float_as_uint(m.x), __float_as_uint(m.y), __float_as_uint(m.z), __float_as_uint(m.w),
                 bh[2 * ks], bh[2 * ks + 1]);
        mma_tf32(q, h0, h1, h2, h3, bm[2 * ks], bm[2 * ks + 1]);
        mma_tf32(acc, h0, h1, h2, h3, bh[2 * ks], bh[2 * ks + 1]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] += p[i] + q[i];
}

// Two m-tiles (mt, mt + 1) at once: six independent accumulation chains (per
// tile: mid x hi, hi x mid, hi x hi), so dependent MMAs issue six apart.
template <int D>
__device__ __forceinline__ void mma_tile2(const float4* __restrict__ frag, uint32_t mt, uint32_t lane,
                                          const uint32_t (&bh)[D / 4], const uint32_t (&bm)[D / 4], float (&acc0)[4],
                                          float (&acc1)[4]) {
    constexpr uint32_t KS = D / 8;
    float p0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, p1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float q0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, q1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 4; ++i) acc0[i] = acc1[i] = 0.0f;
#pragma unroll
    for (uint32_t ks = 0; ks < KS; ++ks) {
        const float4 h = frag[mma_frag_index(mt, ks, 0, lane, KS)];
        const float4 m = frag[mma_frag_index(mt, ks, 1, lane, KS)];
        const float4 h_ = frag[mma_frag_index(mt + 1, ks, 0, lane, KS)];
        const float4 m_ = frag[mma_frag_index(mt + 1, ks, 1, lane, KS)];
        mma_tf32(p0, __float_as_uint(m.x), __float_as_uint(m.y), __float_as_uint(m.z), __float_as_uint(m.w),
                 bh[2 * ks], bh[2 * ks + 1]);
        mma_tf32(p1, __float_as_uint(m_.x), __float_as_uint(m_.y), __float_as_uint(m_.z), __float_as_uint(m_.w),
                 bh[2 * ks], bh[2 * ks + 1]);
        mma_tf32(q0, __float_as_uint(h.x), __float_as_uint(h.y), __float_as_uint(h.z), __float_as_uint(h.w),
                 bm[2 * ks], bm[2 * ks + 1]);
        mma_tf32(q1, __float_as_uint(h_.x), __float_as_uint(h_.y), __float_as_uint(h_.z), __float_as_uint(h_.w),
                 bm[2 * ks], bm[2 * ks + 1]);
        mma_tf32(acc0, __float_as_uint(h.x), __float_as_uint(h.y), __float_as_uint(h.z), __float_as_uint(h.w),
                 bh[2 * ks], bh[2 * ks + 1]);
        mma_tf32(acc1, __float_as_uint(h_.x), __float_as_uint(h_.y), __float_as_uint(h_.z), __float_as_uint(h_.w),
                 bh[2 * ks], bh[2 * ks + 1]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        acc0[i] += p0[i] + q0[i];
        acc1[i] += p1[i] + q1[i];
    }
}

// Scores of one m-tile into the two points' (m1, m2, i1) states.
__device__ __forceinline__ void mma_track(const float (&acc)[4], const float* __restrict__ cn, uint32_t mt,
                                          uint32_t g, float& m1a, float& m2a, uint32_t& i1a, float& m1b, float& m2b,
                                          uint32_t& i1b) {
    const uint32_t c0 = mt * 16 + g, c1 = c0 + 8;
    const float n0 = cn[c0], n1 = cn[c1];
    screen_track(fmaf(-2.0f, acc[0], n0), c0, m1a, m2a, i1a);
    screen_track(fmaf(-2.0f, acc[1], n0), c0, m1b, m2b, i1b);
    screen_track(fmaf(-2.0f, acc[2], n1), c1, m1a, m2a, i1a);
    screen_track(fmaf(-2.0f, acc[3], n1), c1, m1b, m2b, i1b);
}

// Exact reference distance of point p to cluster c (sequential fma chain).
template <int D>
__device__ __forceinline__ float exact_distance(const float* __restrict__ P, uint64_t n, uint64_t p,
                                                const float4* frag, uint32_t c) {
    float acc = 0.0f;
#pragma unroll 4
    for (uint32_t f = 0; f < (uint32_t)D; ++f) {
        const float t = __ldg(P + (size_t)f * n + p) - mma_centroid<D>(frag, c, f);
        acc = f == 0 ? t * t : fmaf(t, t, acc);
    }
    return acc;
}

// Candidate pass for points the bound did not prove but whose values are
// finite (r^2 < 2^120, m1 finite): every cluster whose score is above
// m1 + T is proved farther (in the reference's arithmetic) than the cluster
// of m1, so the reference's label is the lexicographic (distance, index)
// minimum over the candidates (score <= m1 + T), which the lanes holding
// those scores compute exactly.  The MMAs are re-run (same operands, same
// scores).  Returns the labels of points 2t / 2t + 1 (valid where requested).
template <int D>
__device__ __forceinline__ void mma_candidates(const float* __restrict__ P, uint64_t n, uint64_t p0,
                                               const float4* __restrict__ frag, const float* __restrict__ cn,
                                               uint32_t k, const uint32_t (&bh)[D / 4], const uint32_t (&bm)[D / 4],
                                               bool want_a, float lim_a, bool want_b, float lim_b, uint32_t& la,
                                               uint32_t& lb) {
    const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
    float da = INFINITY, db = INFINITY;
    uint32_t ca = 0xffffffffu, cb = 0xffffffffu;
    const uint32_t MT = mma_k_pad(k) >> 4;
#pragma unroll 1
    for (uint32_t mt = 0; mt < MT; ++mt) {
        float acc[4];
        mma_tile<D>(frag, mt, lane, bh, bm, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t c = mt * 16 + g + ((i & 2) ? 8u : 0u);
            const bool is_a = (i & 1) == 0;
            const float sc = fmaf(-2.0f, acc[i], cn[c]);
            if (is_a ? (want_a && sc <= lim_a) : (want_b && sc <= lim_b)) {
                const float dist = exact_distance<D>(P, n, p0 + 2 * t + (is_a ? 0u : 1u), frag, c);
                if (is_a) {
                    if (dist < da || (dist == da && c < ca)) { da = dist; ca = c; }
                } else {
                    if (dist < db || (dist == db && c < cb)) { db = dist; cb = c; }
                }
            }
        }
    }
#pragma unroll
    for (int o = 4; o <= 16; o <<= 1) {
        float od = __shfl_xor_sync(0xffffffffu, da, o);
        uint32_t oc = __shfl_xor_sync(0xffffffffu, ca, o);
        if (od < da || (od == da && oc < ca)) { da = od; ca = oc; }
        od = __shfl_xor_sync(0xffffffffu, db, o);
        oc = __shfl_xor_sync(0xffffffffu, cb, o);
        if (od < db || (od == db && oc < cb)) { db = od; cb = oc; }
    }
    if (want_a) la = ca;
    if (want_b) lb = cb;
}

// Labels 8 points p0 .. p0 + 7 (those < p_end) of a column-major point set
// with the MMA screen; the whole warp calls it.  Lane (g = lane / 4,
// t = lane % 4) holds features 8 ks + t and 8 ks + t + 4 of point p0 + g, split
// as x = hi + mid (exactly; hi + mid in FP32 gives x back) in bh / bm
// [2 ks], [2 ks + 1] (zero for points >= p_end), and on return lab_own is the
// label of point p0 + g.
template <int D>
__device__ __forceinline__ void mma_label8(const float* __restrict__ P, uint64_t n, uint64_t p0, uint64_t p_end,
                                           const float4* __restrict__ frag, const float* __restrict__ cn, float cm,
                                           uint32_t k, uint32_t (&bh)[D / 4], uint32_t (&bm)[D / 4],
                                           uint32_t& lab_own) {
    const uint32_t lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
    const uint64_t pg = p0 + g;
    const bool vg = pg < p_end;
    float nx = 0.0f;
#pragma unroll
    for (uint32_t i = 0; i < D / 4; ++i) {
        const uint32_t f = (i >> 1) * 8 + t + ((i & 1u) ? 4u : 0u);
        const float x = vg ? __ldg(P + (size_t)f * n + pg) : 0.0f;
        bh[i] = to_tf32(x);
        bm[i] = __float_as_uint(x - __uint_as_float(bh[i]));
        nx = fmaf(x, x, nx);
    }
    nx += __shfl_xor_sync(0xffffffffu, nx, 1);
    nx += __shfl_xor_sync(0xffffffffu, nx, 2);  // |x|^2 of point g in its four lanes

    // this lane scores points 2t and 2t + 1 against clusters 16 mt + g and
    // 16 mt + g + 8
    float m1a = INFINITY, m2a = INFINITY, m1b = INFINITY, m2b = INFINITY;
    uint32_t i1a = 0, i1b = 0;
    const uint32_t MT = mma_k_pad(k) >> 4;
    uint32_t mt = 0;
#pragma unroll 1
    for (; mt + 2 <= MT; mt += 2) {
        float acc0[4], acc1[4];
        mma_tile2<D>(frag, mt, lane, bh, bm, acc0, acc1);
        mma_track(acc0, cn, mt, g, m1a, m2a, i1a, m1b, m2b, i1b);
        mma_track(acc1, cn, mt + 1, g, m1a, m2a, i1a, m1b, m2b, i1b);
    }
    if (mt < MT) {
        float acc[4];
        mma_tile<D>(frag, mt, lane, bh, bm, acc);
        mma_track(acc, cn, mt, g, m1a, m2a, i1a, m1b, m2b, i1b);
    }
#pragma unroll
    for (int o = 4; o <= 16; o <<= 1) {
        float a = __shfl_xor_sync(0xffffffffu, m1a, o), b = __shfl_xor_sync(0xffffffffu, m2a, o);
        uint32_t i = __shfl_xor_sync(0xffffffffu, i1a, o);
        screen_merge(m1a, m2a, i1a, a, b, i);
        a = __shfl_xor_sync(0xffffffffu, m1b, o);
        b = __shfl_xor_sync(0xffffffffu, m2b, o);
        i = __shfl_xor_sync(0xffffffffu, i1b, o);
        screen_merge(m1b, m2b, i1b, a, b, i);
    }
    // |x|^2 of points 2t and 2t + 1 from their lanes
    const float nxa = __shfl_sync(0xffffffffu, nx, (2 * t) * 4);
    const float nxb = __shfl_sync(0xffffffffu, nx, (2 * t + 1) * 4);
    constexpr float A = ((float)(D + 8) * 0x1p-22f + (float)(2 * D + 8) * 0x1p-24f) * 1.001f;
    const float ra = (sqrtf(nxa) * (1.0f + 0x1p-16f) + cm) * (1.0f + 0x1p-20f);
    const float rb = (sqrtf(nxb) * (1.0f + 0x1p-16f) + cm) * (1.0f + 0x1p-20f);
    const float Ta = fmaf(A * ra, ra, 0x1p-117f * (ra + 1.0f));
    const float Tb = fmaf(A * rb, rb, 0x1p-117f * (rb + 1.0f));
    const bool va = p0 + 2 * t < p_end, vb = p0 + 2 * t + 1 < p_end;
    // finite: the bound holds, so the candidates decide; else the full pass
    const bool fin_a = (m1a < INFINITY) && (ra * ra < 0x1p120f) && (Ta < INFINITY);
    const bool fin_b = (m1b < INFINITY) && (rb * rb < 0x1p120f) && (Tb < INFINITY);
    const bool ok_a = !va || (fin_a && (m2a - m1a > Ta));
    const bool ok_b = !vb || (fin_b && (m2b - m1b > Tb));
    uint32_t la = i1a, lb = i1b;
    const bool cand_a = !ok_a && fin_a, cand_b = !ok_b && fin_b;
    if (__any_sync(0xffffffffu, cand_a || cand_b))
        mma_candidates<D>(P, n, p0, frag, cn, k, bh, bm, cand_a, m1a + Ta, cand_b, m1b + Tb, la, lb);
    // full exact pass for the rest (lanes 0..3 report points 2t and 2t + 1)
    uint32_t todo = __ballot_sync(0xffffffffu, g == 0 && !ok_a && !fin_a) |
                    (__ballot_sync(0xffffffffu, g == 0 && !ok_b && !fin_b) << 4);
    while (todo) {
        const uint32_t bit = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t pi = bit < 4 ? 2 * bit : 2 * (bit - 4) + 1;
        const uint32_t l = warp_exact_label<D>(P, n, p0 + pi, frag, k, lane);
        if (pi == 2 * t) la = l;
        if (pi == 2 * t + 1) lb = l;
    }
    // the label of this lane's own point g, from lane g / 2 (t = g / 2)
    const uint32_t oa = __shfl_sync(0xffffffffu, la, g >> 1);
    const uint32_t ob = __shfl_sync(0xffffffffu, lb, g >> 1);
    lab_own = (g & 1u) ? ob : oa;
}

}  // namespace ckm
