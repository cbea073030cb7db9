// Device-side helpers shared by the kernels: packed FP32x2 arithmetic,
// warp reductions and the FP64 scratch finalisation every fused / centroid
// update launch ends with.
#pragma once

#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "ckm_internal.h"

namespace ckm {

// --- packed FP32x2 (sm_100 family): two IEEE round-to-nearest operations per
// instruction.  Each lane of the pair rounds exactly like the scalar op, so
// the distance keeps the reference's fma(t, t, acc) bit pattern.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rr;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rr, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rr;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rr, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rc, rr;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rr, ra, rb, rc;\n\t"
        "mov.b64 {%0, %1}, rr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}

__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rr;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rr, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// Three-input minimum (sm_100 family): NaN inputs are ignored like in the
// two-input form, so a NaN distance never becomes the minimum.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// One argmin step over two clusters (c, c + 1) with distances a, b, with the
// reference's rule (strict '<' against the running best, lowest index on a
// tie, NaN never wins): 5 ALU operations for two clusters instead of 6.
__device__ __forceinline__ void argmin_step2(float& best, uint32_t& lab, float a, float b, uint32_t c) {
    const float m = fmin3(best, a, b);
    const uint32_t cand = (a == m) ? c : c + 1u;
    lab = (m < best) ? cand : lab;
    best = m;
}

// VW consecutive floats from shared memory in one access (VW = 4 needs a
// 16-byte aligned address, VW = 2 an 8-byte aligned one).
template <int VW>
__device__ __forceinline__ void load_shared_vec(float* dst, const float* src) {
    if constexpr (VW == 4) {
        const float4 v = *reinterpret_cast<const float4*>(src);
        dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; dst[3] = v.w;
    } else if constexpr (VW == 2) {
        const float2 v = *reinterpret_cast<const float2*>(src);
        dst[0] = v.x; dst[1] = v.y;
    } else {
        dst[0] = *src;
    }
}

// Exact label of one point held in registers against k centroid rows
// cs[c * D + f] in shared memory (row starts 16-byte aligned when D % 4 == 0),
// with the reference's arithmetic: t = x_f - c_f, acc = fma(t, t, acc) in
// feature order, strict '<' argmin from FLT_MAX and cluster 0
// (kmeans_naive.cpp:48-63, lloyd_fused_feature_sum.cl:213-239).  Four clusters
// run per step as independent accumulation chains, so the FMA latency of one
// chain hides behind the other three, and one vector load brings four
// features of a row.  The argmin consumes the four distances in cluster
// order, which gives the sequential scan's result.
template <int D>
__device__ __forceinline__ uint32_t label_rows_exact(const float (&x)[D], const float* __restrict__ cs, uint32_t k) {
    constexpr int VW = (D % 4 == 0) ? 4 : ((D % 2 == 0) ? 2 : 1);
    constexpr int CB = 4;
    float best = FLT_MAX;
    uint32_t lab = 0;
    uint32_t c = 0;
    for (; c + CB <= k; c += CB) {
        const float* r = cs + (size_t)c * D;
        float acc[CB];
#pragma unroll
        for (int f = 0; f < D; f += VW) {
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                float cv[VW];
                load_shared_vec<VW>(cv, r + j * D + f);
#pragma unroll
                for (int v = 0; v < VW; ++v) {
                    const float t = x[f + v] - cv[v];
                    acc[j] = (f + v == 0) ? t * t : fmaf(t, t, acc[j]);
                }
            }
        }
        argmin_step2(best, lab, acc[0], acc[1], c);
        argmin_step2(best, lab, acc[2], acc[3], c + 2u);
    }
    for (; c < k; ++c) {
        const float* r = cs + (size_t)c * D;
        float acc = 0.0f;
#pragma unroll
        for (int f = 0; f < D; f += VW) {
            float cv[VW];
            load_shared_vec<VW>(cv, r + f);
#pragma unroll
            for (int v = 0; v < VW; ++v) {
                const float t = x[f + v] - cv[v];
                acc = (f + v == 0) ? t * t : fmaf(t, t, acc);
            }
        }
        if (acc < best) {
            best = acc;
            lab = c;
        }
    }
    return lab;
}

// label_rows_exact for two points at once: each centroid row is read once
// for both, and the two points' chains run side by side.  Each point gets
// the arithmetic and the scan order of label_rows_exact.
template <int D>
__device__ __forceinline__ void label_rows_exact2(const float (&xa)[D], const float (&xb)[D],
                                                  const float* __restrict__ cs, uint32_t k, uint32_t& la,
                                                  uint32_t& lb) {
    constexpr int VW = (D % 4 == 0) ? 4 : ((D % 2 == 0) ? 2 : 1);
    constexpr int CB = 4;
    float besta = FLT_MAX, bestb = FLT_MAX;
    la = 0;
    lb = 0;
    uint32_t c = 0;
    for (; c + CB <= k; c += CB) {
        const float* r = cs + (size_t)c * D;
        float acca[CB], accb[CB];
#pragma unroll
        for (int f = 0; f < D; f += VW) {
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                float cv[VW];
                load_shared_vec<VW>(cv, r + j * D + f);
#pragma unroll
                for (int v = 0; v < VW; ++v) {
                    const float ta = xa[f + v] - cv[v];
                    const float tb = xb[f + v] - cv[v];
                    acca[j] = (f + v == 0) ? ta * ta : fmaf(ta, ta, acca[j]);
                    accb[j] = (f + v == 0) ? tb * tb : fmaf(tb, tb, accb[j]);
                }
            }
        }
        argmin_step2(besta, la, acca[0], acca[1], c);
        argmin_step2(besta, la, acca[2], acca[3], c + 2u);
        argmin_step2(bestb, lb, accb[0], accb[1], c);
        argmin_step2(bestb, lb, accb[2], accb[3], c + 2u);
    }
    for (; c < k; ++c) {
        const float* r = cs + (size_t)c * D;
        float acca = 0.0f, accb = 0.0f;
#pragma unroll
        for (int f = 0; f < D; f += VW) {
            float cv[VW];
            load_shared_vec<VW>(cv, r + f);
#pragma unroll
            for (int v = 0; v < VW; ++v) {
                const float ta = xa[f + v] - cv[v];
                const float tb = xb[f + v] - cv[v];
                acca = (f + v == 0) ? ta * ta : fmaf(ta, ta, acca);
                accb = (f + v == 0) ? tb * tb : fmaf(tb, tb, accb);
            }
        }
        if (acca < besta) {
            besta = acca;
            la = c;
        }
        if (accb < bestb) {
            bestb = accb;
            lb = c;
        }
    }
}

// Certified screen in front of label_rows_exact (D % 4 == 0).
//
// Score s_c = |c|^2 - 2 x.c: the dot product runs as two packed FP32 chains
// (even and odd features, one FFMA2 per feature pair), then
// s_c = fma(-2, dot, cn[c]); half the FMA-pipe work of the exact distance and
// a third of its instructions.  The screen keeps the lowest score m1
// (cluster c1) and the second lowest m2.  With r >= |x| + max_c |c|,
//   |s_c(computed) - s_c(exact)|            <= B   = (D/2 + 4) u r^2,
//   |reference distance - exact distance|   <= rho * exact, rho = (D + 4) u,
// (u = 2^-24; reference distance = the sequential t = x - c, fma(t, t, acc)
// chain, exact distance = |x|^2 + s_c in real arithmetic), so
// m2 - m1 > T = 2B + 2 rho r^2 = (3D + 16) u r^2 proves that the reference's
// distance to c1 is strictly below its distance to every other cluster: the
// reference's strict '<' scan then returns c1.  T is taken as
// (4D + 32) u r^2 (1.001) + 2^-126 (margin for the rounding of r and T and for
// underflow).  A point that is not proved that way (near ties, exact ties,
// NaN or infinite scores, r^2 >= 2^120 where the reference's distances could
// reach FLT_MAX) gets label_rows_exact.  NaN centroids (cn = NaN) never
// become m1 or m2, as they never win in the reference.
//
// cs: centroid rows [c * D + f] (16-byte aligned rows); cn[c] = |c|^2 rounded
// once to FP32 (NaN for a NaN centroid); cm >= max |c| over the non-NaN
// centroids (infinite if a centroid is infinite).
__device__ __forceinline__ void screen_track(float s, uint32_t c, float& m1, float& m2, uint32_t& i1) {
    const bool lt = s < m1;
    m2 = lt ? m1 : fminf(m2, s);
    i1 = lt ? c : i1;
    m1 = lt ? s : m1;
}

template <int D>
__device__ __forceinline__ uint32_t label_rows_screened(const float (&x)[D], const float* __restrict__ cs,
                                                        const float* __restrict__ cn, float cm, uint32_t k) {
    static_assert(D % 4 == 0, "screened rows need D % 4 == 0");
    constexpr int CB = 4;
    float2 nx = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int f = 0; f < D; f += 2) nx = fma2(make_float2(x[f], x[f + 1]), make_float2(x[f], x[f + 1]), nx);
    const float xn = sqrtf(nx.x + nx.y) * (1.0f + 0x1p-16f);
    const float r = (xn + cm) * (1.0f + 0x1p-20f);
    const float T = fmaf((float)(4 * D + 32) * 0x1p-24f * r, r, 0x1p-126f) * 1.001f;

    float m1 = INFINITY, m2 = INFINITY;
    uint32_t i1 = 0;
    uint32_t c = 0;
    for (; c + CB <= k; c += CB) {
        const float* row = cs + (size_t)c * D;
        float2 acc[CB];
#pragma unroll
        for (int j = 0; j < CB; ++j) acc[j] = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int f = 0; f < D; f += 4) {
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                const float4 v = *reinterpret_cast<const float4*>(row + j * D + f);
                acc[j] = fma2(make_float2(x[f], x[f + 1]), make_float2(v.x, v.y), acc[j]);
                acc[j] = fma2(make_float2(x[f + 2], x[f + 3]), make_float2(v.z, v.w), acc[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < CB; ++j) screen_track(fmaf(-2.0f, acc[j].x + acc[j].y, cn[c + j]), c + j, m1, m2, i1);
    }
    for (; c < k; ++c) {
        const float* row = cs + (size_t)c * D;
        float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int f = 0; f < D; f += 4) {
            const float4 v = *reinterpret_cast<const float4*>(row + f);
            acc = fma2(make_float2(x[f], x[f + 1]), make_float2(v.x, v.y), acc);
            acc = fma2(make_float2(x[f + 2], x[f + 3]), make_float2(v.z, v.w), acc);
        }
        screen_track(fmaf(-2.0f, acc.x + acc.y, cn[c]), c, m1, m2, i1);
    }
    const bool proved = (m1 < INFINITY) && (m2 - m1 > T) && (r * r < 0x1p120f);
    if (proved) return i1;
    return label_rows_exact<D>(x, cs, k);
}

// label_rows_screened for two points at once (each centroid row read once
// for both); an unproved point gets label_rows_exact on its own.
template <int D>
__device__ __forceinline__ void label_rows_screened2(const float (&xa)[D], const float (&xb)[D],
                                                     const float* __restrict__ cs, const float* __restrict__ cn,
                                                     float cm, uint32_t k, uint32_t& la, uint32_t& lb) {
    static_assert(D % 4 == 0, "screened rows need D % 4 == 0");
    constexpr int CB = 4;
    float2 nxa = make_float2(0.0f, 0.0f), nxb = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int f = 0; f < D; f += 2) {
        nxa = fma2(make_float2(xa[f], xa[f + 1]), make_float2(xa[f], xa[f + 1]), nxa);
        nxb = fma2(make_float2(xb[f], xb[f + 1]), make_float2(xb[f], xb[f + 1]), nxb);
    }
    const float ra = (sqrtf(nxa.x + nxa.y) * (1.0f + 0x1p-16f) + cm) * (1.0f + 0x1p-20f);
    const float rb = (sqrtf(nxb.x + nxb.y) * (1.0f + 0x1p-16f) + cm) * (1.0f + 0x1p-20f);
    const float Ta = fmaf((float)(4 * D + 32) * 0x1p-24f * ra, ra, 0x1p-126f) * 1.001f;
    const float Tb = fmaf((float)(4 * D + 32) * 0x1p-24f * rb, rb, 0x1p-126f) * 1.001f;

    float m1a = INFINITY, m2a = INFINITY, m1b = INFINITY, m2b = INFINITY;
    uint32_t i1a = 0, i1b = 0;
    uint32_t c = 0;
    for (; c + CB <= k; c += CB) {
        const float* row = cs + (size_t)c * D;
        float2 acca[CB], accb[CB];
#pragma unroll
        for (int j = 0; j < CB; ++j) {
            acca[j] = make_float2(0.0f, 0.0f);
            accb[j] = make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int f = 0; f < D; f += 4) {
#pragma unroll
            for (int j = 0; j < CB; ++j) {
                const float4 v = *reinterpret_cast<const float4*>(row + j * D + f);
                acca[j] = fma2(make_float2(xa[f], xa[f + 1]), make_float2(v.x, v.y), acca[j]);
                acca[j] = fma2(make_float2(xa[f + 2], xa[f + 3]), make_float2(v.z, v.w), acca[j]);
                accb[j] = fma2(make_float2(xb[f], xb[f + 1]), make_float2(v.x, v.y), accb[j]);
                accb[j] = fma2(make_float2(xb[f + 2], xb[f + 3]), make_float2(v.z, v.w), accb[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < CB; ++j) {
            screen_track(fmaf(-2.0f, acca[j].x + acca[j].y, cn[c + j]), c + j, m1a, m2a, i1a);
            screen_track(fmaf(-2.0f, accb[j].x + accb[j].y, cn[c + j]), c + j, m1b, m2b, i1b);
        }
    }
    for (; c < k; ++c) {
        const float* row = cs + (size_t)c * D;
        float2 acca = make_float2(0.0f, 0.0f), accb = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int f = 0; f < D; f += 4) {
            const float4 v = *reinterpret_cast<const float4*>(row + f);
            acca = fma2(make_float2(xa[f], xa[f + 1]), make_float2(v.x, v.y), acca);
            acca = fma2(make_float2(xa[f + 2], xa[f + 3]), make_float2(v.z, v.w), acca);
            accb = fma2(make_float2(xb[f], xb[f + 1]), make_float2(v.x, v.y), accb);
            accb = fma2(make_float2(xb[f + 2], xb[f + 3]), make_float2(v.z, v.w), accb);
        }
        screen_track(fmaf(-2.0f, acca.x + acca.y, cn[c]), c, m1a, m2a, i1a);
        screen_track(fmaf(-2.0f, accb.x + accb.y, cn[c]), c, m1b, m2b, i1b);
    }
    la = ((m1a < INFINITY) && (m2a - m1a > Ta) && (ra * ra < 0x1p120f)) ? i1a : label_rows_exact<D>(xa, cs, k);
    lb = ((m1b < INFINITY) && (m2b - m1b > Tb) && (rb * rb < 0x1p120f)) ? i1b : label_rows_exact<D>(xb, cs, k);
}

// Prologue of the screen, run by every thread of a CTA after the centroid rows
// are in shared memory (and followed by a barrier before use): cn[c] = |c|^2
// (FP64 sum, one rounding) and the maximum of the non-NaN cn into *s_cn_max
// (as float bits, which order like the non-negative floats; zero it first).
__device__ __forceinline__ void screen_norms(const float* __restrict__ cs, uint32_t d, uint32_t k, float* cn,
                                             unsigned int* s_cn_max, uint32_t tid, uint32_t nthreads) {
    for (uint32_t c = tid; c < k; c += nthreads) {
        const float* row = cs + (size_t)c * d;
        double s = 0.0;
        for (uint32_t f = 0; f < d; ++f) s = fma((double)row[f], (double)row[f], s);
        const float v = (float)s;
        cn[c] = v;
        if (!isnan(v)) atomicMax(s_cn_max, __float_as_uint(v));
    }
}

// cm >= max |c| from the maximum squared norm (rounded up).
__device__ __forceinline__ float screen_cm(unsigned int cn_max_bits) {
    return sqrtf(__uint_as_float(cn_max_bits)) * (1.0f + 0x1p-16f);
}

__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Type maximum used as the argmin's starting value (the reference's
// CL_POINT_MAX / std::numeric_limits<PointT>::max()).
template <typename T> struct TypeMax;
template <> struct TypeMax<float> { static __device__ __forceinline__ float v() { return FLT_MAX; } };
template <> struct TypeMax<double> { static __device__ __forceinline__ double v() { return DBL_MAX; } };

// Takes a ticket after this CTA merged its partials; returns true in the one
// CTA that arrives last (all other CTAs' FP64 atomics are then visible).
__device__ __forceinline__ bool last_cta_ticket(unsigned int* counter) {
    __shared__ unsigned int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(counter, 1u);
        s_last = (t == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    bool last = s_last != 0;
    if (last) __threadfence();
    return last;
}

// Turns the FP64 scratch into the call's outputs and re-zeroes it.
//   FINALIZE:   C = sums / masses (0/0 -> NaN), masses = counts
//   ACCUMULATE: C += sums, masses += counts      (reference functor contract)
// Run by every thread of one CTA.
template <typename T, typename M>
__device__ void finalize_block(uint32_t d, uint32_t k, T* C, M* masses, ScratchView sv, int mode) {
    const uint64_t kd = (uint64_t)k * d;
    for (uint64_t e = threadIdx.x; e < kd; e += blockDim.x) {
        const uint32_t c = (uint32_t)(e % k);
        const double s = __ldcg(&sv.sums[e]);
        if (mode == CKM_MODE_FINALIZE) {
            const double m = (double)__ldcg(&sv.masses[c]);
            C[e] = (T)(s / m);
        } else {
            C[e] = C[e] + (T)s;
        }
        sv.sums[e] = 0.0;
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) {
        const unsigned long long m = __ldcg(&sv.masses[c]);
        if (masses != nullptr) {  // the centroid-update pass leaves masses alone
            if (mode == CKM_MODE_FINALIZE) masses[c] = (M)m;
            else masses[c] = masses[c] + (M)m;
        }
        sv.masses[c] = 0ull;
    }
    if (threadIdx.x == 0) sv.ctrl[0] = 0u;
}

}  // namespace ckm
