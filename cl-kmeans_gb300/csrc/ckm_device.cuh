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
