// Batched Lloyd iterations: many independent k-means jobs of uneven n, d and
// k in ONE persistent launch per iteration.
//
// The host cuts every job into tiles of `tile` points and groups contiguous
// runs of tiles ("segments", never spanning two jobs) into units of similar
// estimated cost, listed largest first.  The CTAs claim segments from a
// counter until none are left (dynamic scheduling: a static split by
// estimated cost left most SMs idle behind a few slow CTAs, because small-k
// jobs pay for shared-memory atomic contention that the estimate does not
// see).  Per segment a CTA stages the job's centroids in shared memory,
// labels each point with the reference's result (fma(t,t,acc) over the
// features, strict '<' argmin from cluster 0; kmeans_naive.cpp:48-63): the
// exact loop for d = 2 / 4, a certified FP32 screen in front of it for
// d >= 8, and for d = 32 / 64 a certified tensor-core screen (the tcgen05 path
// of ckm_umma_batch.cuh in 512-thread CTAs, else TF32 mma.sync), and adds each
// point into a shared-memory sum/mass table, which it merges into the job's
// FP64 scratch every `flush` tiles and at the end of the segment.  Each job
// carries a tile ticket: the CTA whose merge completes the job's tiles
// finalises that job (centroids = sums / masses into the other buffer of the
// job's centroid pair, masses, relative centroid shift) and re-zeroes its
// scratch.  Nothing waits on another CTA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ckm_batched.h"
#include "ckm_device.cuh"
#include "ckm_internal.h"
#include "ckm_mma_screen.cuh"
#include "ckm_umma_batch.cuh"

namespace ckm {

namespace {

// threads per CTA: 256 (two or more CTAs per SM) or 512 (one CTA per SM
// with the whole shared memory, so the largest tables stay on chip)

// Shared memory per CTA: centroids [c][f] (if they fit) + sum table [f][c] +
// mass table [c].
template <int BT>
__device__ __forceinline__ void stage_centroids(const BatchJobDev& J, const float* __restrict__ src, float* s_c,
                                                bool cent_smem) {
    if (!cent_smem) return;
    const uint32_t k = J.k, d = J.d;
    for (uint32_t i = threadIdx.x; i < k * d; i += BT) {
        const uint32_t c = i / d, f = i - c * d;
        s_c[i] = src[(size_t)f * k + c];
    }
}

__device__ __forceinline__ uint32_t label_point_generic(const float* __restrict__ P, uint64_t n, uint64_t p,
                                                        const float* __restrict__ cs, bool cent_smem,
                                                        const float* __restrict__ gc, uint32_t k, uint32_t d) {
    float best = FLT_MAX;
    uint32_t lab = 0;
    for (uint32_t c = 0; c < k; ++c) {
        float acc = 0.f;
        for (uint32_t f = 0; f < d; ++f) {
            const float cf = cent_smem ? cs[(size_t)c * d + f] : __ldg(gc + (size_t)f * k + c);
            const float t = __ldg(P + (size_t)f * n + p) - cf;
            acc = fmaf(t, t, acc);
        }
        if (acc < best) {
            best = acc;
            lab = c;
        }
    }
    return lab;
}

// The job's centroid buffer `parity`: a select, not an indexed access, so the
// job record stays in registers (an indexed member would put it on the stack).
__device__ __forceinline__ float* cent_of(const BatchJobDev& J, int parity) {
    return parity ? J.cent[1] : J.cent[0];
}

// Where a segment adds its points, per job by table size: a shared table of
// `copies` (a power of two up to 32) interleaved copies of the sums,
// s_sum[(f * k + c) * copies + (lane & (copies - 1))], and one mass column
// s_mass[c]; or, with copies = 0, straight into the job's FP64 scratch.  A
// shared-memory FP32 atomic add retries while other lanes of the warp hit the
// same word (eight lanes on one word ran 7.6 times slower than eight words),
// so the copies keep the lanes of a warp apart: with 32 copies they never
// meet.  Integer atomics do not slow down that way, so masses keep one copy.
__device__ __forceinline__ void add_feature(const BatchJobDev& J, float* s_sum, uint32_t copies, uint32_t f,
                                            uint32_t lab, float v) {
    if (copies) atomicAdd(&s_sum[((size_t)f * J.k + lab) * copies + (threadIdx.x & (copies - 1u))], v);
    else atomicAdd(&J.sums[(size_t)f * J.k + lab], (double)v);
}

__device__ __forceinline__ void add_mass(const BatchJobDev& J, unsigned int* s_mass, uint32_t copies, uint32_t lab) {
    if (copies) atomicAdd(&s_mass[lab], 1u);
    else atomicAdd(&J.msum[lab], 1ull);
}

// The most copies (32, 16, ..., 1) whose table fits in `cap` bytes; 0 if none.
__device__ __forceinline__ uint32_t table_copies(uint32_t k, uint32_t d, size_t cap) {
    const size_t kd = (size_t)k * d;
    for (uint32_t c = 32; c >= 1; c >>= 1)
        if ((kd * c + k) * sizeof(float) <= cap) return c;
    return 0;
}

// Labels the points of tiles [t0, t1) of one job and adds them up.
// d = 8, 16, 32, 64 go through the certified screen (label_rows_screened:
// packed dot products, exact fallback per unproved point); d = 2, 4 use the
// exact loop directly.
template <int D> struct Screened { static constexpr bool value = D >= 8 && D % 4 == 0; };

template <int D, int BT>
__device__ __forceinline__ void run_tiles_fixed(const BatchJobDev& J, uint32_t t0, uint32_t t1, uint32_t tile,
                                                const float* s_c, const float* s_cn, float cm, float* s_sum,
                                                unsigned int* s_mass, uint32_t copies) {
    const uint64_t n = J.n;
    const uint32_t k = J.k;
    const float* __restrict__ P = J.points;
    for (uint64_t p = (uint64_t)t0 * tile + threadIdx.x; p < (uint64_t)t1 * tile && p < n; p += BT) {
        float x[D];
#pragma unroll
        for (int f = 0; f < D; ++f) x[f] = __ldg(P + (size_t)f * n + p);
        uint32_t lab;
        if constexpr (Screened<D>::value) lab = label_rows_screened<D>(x, s_c, s_cn, cm, k);
        else lab = label_rows_exact<D>(x, s_c, k);
        J.labels[p] = lab;
#pragma unroll
        for (int f = 0; f < D; ++f) add_feature(J, s_sum, copies, f, lab, x[f]);
        add_mass(J, s_mass, copies, lab);
    }
}

// run_tiles_fixed for D <= 16 with two points per thread (p and p + BT):
// each centroid row read from shared memory serves both, and the two points'
// chains run side by side.  Labels and sums per point as run_tiles_fixed.
template <int D, int BT>
__device__ __forceinline__ void run_tiles_fixed2(const BatchJobDev& J, uint32_t t0, uint32_t t1, uint32_t tile,
                                                 const float* s_c, const float* s_cn, float cm, float* s_sum,
                                                 unsigned int* s_mass, uint32_t copies) {
    const uint64_t n = J.n;
    const uint32_t k = J.k;
    const float* __restrict__ P = J.points;
    const uint64_t hi = min((uint64_t)t1 * tile, n);
    for (uint64_t p = (uint64_t)t0 * tile + threadIdx.x; p < hi; p += 2 * BT) {
        const uint64_t q = p + BT;
        const bool vq = q < hi;
        float xa[D], xb[D];
#pragma unroll
        for (int f = 0; f < D; ++f) {
            xa[f] = __ldg(P + (size_t)f * n + p);
            xb[f] = vq ? __ldg(P + (size_t)f * n + q) : xa[f];
        }
        uint32_t la, lb;
        if constexpr (Screened<D>::value) label_rows_screened2<D>(xa, xb, s_c, s_cn, cm, k, la, lb);
        else label_rows_exact2<D>(xa, xb, s_c, k, la, lb);
        J.labels[p] = la;
#pragma unroll
        for (int f = 0; f < D; ++f) add_feature(J, s_sum, copies, f, la, xa[f]);
        add_mass(J, s_mass, copies, la);
        if (vq) {
            J.labels[q] = lb;
#pragma unroll
            for (int f = 0; f < D; ++f) add_feature(J, s_sum, copies, f, lb, xb[f]);
            add_mass(J, s_mass, copies, lb);
        }
    }
}

template <int BT>
__device__ __forceinline__ void run_tiles_generic(const BatchJobDev& J, uint32_t t0, uint32_t t1, uint32_t tile, const float* s_c,
                                  bool cent_smem, float* s_sum, unsigned int* s_mass, uint32_t copies, int parity) {
    const uint64_t n = J.n;
    const uint32_t k = J.k, d = J.d;
    const float* __restrict__ P = J.points;
    const float* gc = cent_of(J, parity);
    for (uint64_t p = (uint64_t)t0 * tile + threadIdx.x; p < (uint64_t)t1 * tile && p < n; p += BT) {
        const uint32_t lab = label_point_generic(P, n, p, s_c, cent_smem, gc, k, d);
        J.labels[p] = lab;
        for (uint32_t f = 0; f < d; ++f) add_feature(J, s_sum, copies, f, lab, __ldg(P + (size_t)f * n + p));
        add_mass(J, s_mass, copies, lab);
    }
}

// d = 32 / 64 jobs with enough clusters (mma_min_k): 8 points per warp
// through the tensor-core screen (mma_label8), then each lane adds its
// quarter of its point's features into the table.
template <int D, int BT>
__device__ __forceinline__ void run_tiles_mma(const BatchJobDev& J, uint32_t t0, uint32_t t1, uint32_t tile,
                                              const float4* frag, const float* s_cn, float cm, float* s_sum,
                                              unsigned int* s_mass, uint32_t copies) {
    const uint64_t n = J.n;
    const uint32_t k = J.k;
    const uint64_t begin = (uint64_t)t0 * tile;
    const uint64_t end = min((uint64_t)t1 * tile, n);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
#pragma unroll 1
    for (uint64_t p0 = begin + (uint64_t)warp * 8; p0 < end; p0 += (uint64_t)(BT / 32) * 8) {
        uint32_t bh[D / 4], bm[D / 4];
        uint32_t lab;
        mma_label8<D>(J.points, n, p0, end, frag, s_cn, cm, k, bh, bm, lab);
        if (p0 + g < end) {
            if (t == 0) J.labels[p0 + g] = lab;
#pragma unroll
            for (uint32_t i = 0; i < (uint32_t)D / 4; ++i) {
                const uint32_t f = (i >> 1) * 8 + t + ((i & 1u) ? 4u : 0u);
                add_feature(J, s_sum, copies, f, lab, __uint_as_float(bh[i]) + __uint_as_float(bm[i]));  // x exactly
            }
            if (t == 0) add_mass(J, s_mass, copies, lab);
        }
    }
}

// Merges the shared table into the job's FP64 scratch and re-zeroes it.
template <int BT>
__device__ __forceinline__ void flush_tables(const BatchJobDev& J, float* s_sum, unsigned int* s_mass,
                                             uint32_t copies) {
    const uint32_t k = J.k, d = J.d;
    const uint32_t kd = k * d;
    if (copies == 32) {
        // one warp per entry: the 32 copies summed with shuffles
        const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (uint32_t e = warp; e < kd; e += BT / 32) {
            float v = s_sum[(size_t)e * 32 + lane];
            s_sum[(size_t)e * 32 + lane] = 0.f;
            v = warp_sum_f32(v);
            if (lane == 0 && v != 0.f) atomicAdd(&J.sums[e], (double)v);
        }
    } else {
        for (uint32_t e = threadIdx.x; e < kd; e += BT) {
            float* src = s_sum + (size_t)e * copies;
            float v = 0.f;
            for (uint32_t j = 0; j < copies; ++j) {
                v += src[j];
                src[j] = 0.f;
            }
            if (v != 0.f) atomicAdd(&J.sums[e], (double)v);
        }
    }
    for (uint32_t c = threadIdx.x; c < k; c += BT) {
        const unsigned int m = s_mass[c];
        if (m) atomicAdd(&J.msum[c], (unsigned long long)m);
        s_mass[c] = 0u;
    }
}

// Last CTA of a job: centroids, masses, relative shift; scratch back to zero.
template <int BT>
__device__ __forceinline__ void finalize_job(const BatchJobDev& J, int parity, float tol, uint32_t max_it) {
    __shared__ float s_red[BT / 32 * 2];
    const uint32_t k = J.k, d = J.d;
    const float* old = cent_of(J, parity);
    float* out = cent_of(J, parity ^ 1);
    float dmax = 0.f, cmax = 0.f;
    for (uint32_t e = threadIdx.x; e < k * d; e += BT) {
        const uint32_t c = e % k;
        const double s = __ldcg(&J.sums[e]);
        const double m = (double)__ldcg(&J.msum[c]);
        const float v = (float)(s / m);
        const float o = old[e];
        out[e] = v;
        dmax = fmaxf(dmax, fabsf(v - o));  // NaN (empty cluster) is ignored by fmaxf
        cmax = fmaxf(cmax, fabsf(o));
        J.sums[e] = 0.0;
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < k; c += BT) {
        J.masses[c] = (uint32_t)__ldcg(&J.msum[c]);
        J.msum[c] = 0ull;
    }
    for (int o = 16; o > 0; o >>= 1) {
        dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_red[threadIdx.x >> 5] = dmax;
        s_red[BT / 32 + (threadIdx.x >> 5)] = cmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < BT / 32; ++w) {
            a = fmaxf(a, s_red[w]);
            b = fmaxf(b, s_red[BT / 32 + w]);
        }
        const float shift = a / fmaxf(b, 1e-30f);
        const uint32_t its = J.status->iterations + 1;
        J.status->shift = shift;
        J.status->iterations = its;
        // convergence stop: the job parks itself (bit 0: skipped by later
        // steps; bit 1: finished) once its shift is below the tolerance or it
        // has run max_it iterations
        if ((tol > 0.f && shift < tol) || (max_it != 0u && its >= max_it)) J.status->flags |= 3u;
        J.status->parity = (uint32_t)(parity ^ 1);
        *J.ticket = 0u;
    }
}

template <int BT>
__global__ void __launch_bounds__(BT, 512 / BT) batched_kernel(const BatchJobDev* __restrict__ jobs,
                                                     const BatchSegment* __restrict__ segs, uint32_t num_segs,
                                                     unsigned int* __restrict__ work, float tol, uint32_t max_it,
                                                     uint32_t tile,
                                                     uint32_t flush_tiles, size_t cent_cap, size_t acc_cap,
                                                     uint32_t use_umma) {
    // use_umma bit 0: the tcgen05 path may run; bit 1: failure-detection test
    // (each CTA's first half gives up on its first tensor-core wait)
    const bool umma_test_stall = (use_umma & 2u) != 0u;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned int s_last, s_unit, s_cn_max;
    // tensor-core path: TMEM accumulator, MMA-completion barrier, abort flag
    __shared__ __align__(8) uint64_t s_ubar[2];  // one per CTA half
    __shared__ uint32_t s_tmem;
    __shared__ unsigned int s_abort;
    const uint32_t ubar = umma::smem_u32(&s_ubar[0]);
    const uint32_t ubase = (umma::smem_u32(smem) + 1023u) & ~1023u;
    uint32_t uphase = 0;
    bool aborted = false;
    if (BT == 512 && use_umma) {
        if (threadIdx.x == 0) {
            umma::mbar_init(ubar, 1);
            umma::mbar_init(ubar + 8u, 1);
            umma::mbar_fence_init();
            s_abort = 0u;
        }
        if (threadIdx.x < 32) umma::tmem_alloc(umma::smem_u32(&s_tmem), UMMA_TMEM_COLS);
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    for (;;) {
        // dynamic schedule: the next unclaimed segment (largest first)
        __syncthreads();  // every thread has read the previous s_unit and cm
        if (threadIdx.x == 0) {
            s_unit = atomicAdd(work, 1u);
            s_cn_max = 0u;  // zeroed a barrier before any atomicMax of this segment
        }
        __syncthreads();
        const uint32_t si = s_unit;
        if (si >= num_segs) break;
        const BatchSegment S = segs[si];
        const BatchJobDev J = jobs[S.job];
        // parity and flags were last written by the previous launch (or by the
        // host before it); within a launch only the job's finalising CTA
        // changes them, after every segment of the job has read them
        const BatchStatus st = *J.status;
        if (st.flags & 1u) continue;  // job inactive this step
        const int parity = (int)(st.parity & 1u);
        const uint32_t k = J.k, d = J.d;
        const size_t total = cent_cap + acc_cap;
        // d = 32 / 64 on the tensor cores (tcgen05) when the segment's layout
        // and a one-copy table fit, and the centroids are within fp16's range
        bool umma = BT == 512 && use_umma && (d == 32 || d == 64) && k >= UMMA_MIN_K && k <= UMMA_MAX_K &&
                    umma_region_bytes(k) + ((size_t)k * d + k) * sizeof(float) <= total;
        if constexpr (BT == 512) if (umma) {
            __shared__ UmmaScratch s_us;
            const uint32_t kp = umma_k_pad(k);
            const UmmaLayout L = umma_layout(kp);
            const size_t table_off = umma_region_bytes(k);
            const uint32_t copies = table_copies(k, d, total - table_off);
            float* s_sum = reinterpret_cast<float*>(smem + table_off);
            unsigned int* s_mass = reinterpret_cast<unsigned int*>(s_sum + (size_t)k * d * copies);
            const float* C = cent_of(J, parity);
            __syncthreads();  // previous segment's readers of shared memory are done
            if (d == 32) umma_stage<32, BT>(C, k, ubase, L, kp, s_us.cn, &s_cn_max);
            else umma_stage<64, BT>(C, k, ubase, L, kp, s_us.cn, &s_cn_max);
            {
                const size_t words = (size_t)k * d * copies + k;
                for (size_t i = threadIdx.x; i < words; i += BT) s_sum[i] = 0.f;
            }
            umma::fence_proxy_async_smem();
            __syncthreads();
            const float cm = __uint_as_float(s_cn_max);
            umma = cm < UMMA_MAX_ABS;  // same value in every thread
            if (umma) {
                for (uint32_t t = S.tile_begin; t < S.tile_end && !aborted; t += flush_tiles) {
                    const uint32_t te = min(S.tile_end, t + flush_tiles);
                    const bool ok = d == 32 ? run_tiles_umma<32>(J, C, t, te, tile, ubase, L, kp, s_tmem, ubar, uphase,
                                                                 cm, s_sum, s_mass, copies, s_us, &s_abort,
                                                                 umma_test_stall)
                                            : run_tiles_umma<64>(J, C, t, te, tile, ubase, L, kp, s_tmem, ubar, uphase,
                                                                 cm, s_sum, s_mass, copies, s_us, &s_abort,
                                                                 umma_test_stall);
                    if (!ok) {
                        aborted = true;  // every thread: the flag was read after a barrier
                        break;
                    }
                    if (copies) {
                        __syncthreads();
                        flush_tables<BT>(J, s_sum, s_mass, copies);
                        __syncthreads();
                    }
                }
                if (aborted) {
                    // the job cannot finish this step: parked with the error bit
                    if (threadIdx.x == 0) atomicOr(&J.status->flags, 7u);
                    break;
                }
            }
        }
        if (!umma) {
        // shared memory of this segment: centroids (MMA fragments, or rows for
        // the SIMT screen / exact loop, or none) at the start, the sum table
        // in the rest
        const bool mma = (d == 32 || d == 64) && k >= mma_min_k(d) &&
                         mma_cent_bytes(k, d) + ((size_t)k * d + k) * sizeof(float) <= total;
        const size_t cbytes = ((size_t)k * d + ((k + 3u) & ~3u)) * sizeof(float);  // rows + |c|^2
        const bool cent_smem = !mma && cbytes <= cent_cap;
        const size_t table_off = mma ? mma_cent_bytes(k, d) : (cent_smem ? ((cbytes + 15) & ~size_t(15)) : 0);
        const uint32_t copies = table_copies(k, d, total - table_off);
        float* s_c = reinterpret_cast<float*>(smem);
        float* s_cn = mma ? s_c + (size_t)mma_k_pad(k) * d * 2 : s_c + (size_t)k * d;
        float* s_sum = reinterpret_cast<float*>(smem + table_off);
        unsigned int* s_mass = reinterpret_cast<unsigned int*>(s_sum + (size_t)k * d * copies);
        __syncthreads();  // previous segment's readers of the shared tables are done
        if (mma) {
            if (d == 32) mma_stage_centroids<32>(cent_of(J, parity), k, reinterpret_cast<float4*>(s_c), s_cn, &s_cn_max, threadIdx.x, BT);
            else mma_stage_centroids<64>(cent_of(J, parity), k, reinterpret_cast<float4*>(s_c), s_cn, &s_cn_max, threadIdx.x, BT);
        } else {
            stage_centroids<BT>(J, cent_of(J, parity), s_c, cent_smem);
        }
        {
            const size_t words = copies ? (size_t)k * d * copies + k : 0;
            for (size_t i = threadIdx.x; i < words; i += BT) s_sum[i] = 0.f;  // sums, then masses
        }
        __syncthreads();
        const bool screen = cent_smem && (d == 8 || d == 16 || d == 32 || d == 64);
        if (screen) {
            screen_norms(s_c, d, k, s_cn, &s_cn_max, threadIdx.x, BT);
            __syncthreads();
        }
        const float cm = screen_cm(s_cn_max);
        for (uint32_t t = S.tile_begin; t < S.tile_end; t += flush_tiles) {
            const uint32_t te = min(S.tile_end, t + flush_tiles);
            if (mma) {
                if (d == 32) run_tiles_mma<32, BT>(J, t, te, tile, reinterpret_cast<const float4*>(s_c), s_cn, cm, s_sum, s_mass, copies);
                else run_tiles_mma<64, BT>(J, t, te, tile, reinterpret_cast<const float4*>(s_c), s_cn, cm, s_sum, s_mass, copies);
            } else if (cent_smem) {
                switch (d) {
                    case 2: run_tiles_fixed2<2, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    case 4: run_tiles_fixed2<4, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    case 8: run_tiles_fixed2<8, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    case 16: run_tiles_fixed2<16, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    case 32: run_tiles_fixed<32, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    case 64: run_tiles_fixed<64, BT>(J, t, te, tile, s_c, s_cn, cm, s_sum, s_mass, copies); break;
                    default: run_tiles_generic<BT>(J, t, te, tile, s_c, true, s_sum, s_mass, copies, parity); break;
                }
            } else {
                run_tiles_generic<BT>(J, t, te, tile, s_c, false, s_sum, s_mass, copies, parity);
            }
            if (copies) {
                __syncthreads();
                flush_tables<BT>(J, s_sum, s_mass, copies);
                __syncthreads();
            }
        }
        }
        // ticket: the CTA that completes the job's tiles finalises it
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t mine = S.tile_end - S.tile_begin;
            const unsigned int before = atomicAdd(J.ticket, mine);
            s_last = (before + mine == J.num_tiles) ? 1u : 0u;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            finalize_job<BT>(J, parity, tol, max_it);
        }
    }
    if (BT == 512 && use_umma) {
        // (after an abort each half waited, bounded, for its last MMA)
        umma::fence_before_sync();
        __syncthreads();
        if (threadIdx.x < 32) {
            umma::fence_after_sync();
            umma::tmem_dealloc(s_tmem, UMMA_TMEM_COLS);
        }
    }
}

// Raises the kernel's dynamic shared-memory limit (once per device and CTA
// size) to the opt-in maximum minus its static shared memory.
template <int BT>
int ensure_batched_attr() {
    static bool attr_done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr_done[dev]) {
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, batched_kernel<BT>);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(batched)");
        e = cudaFuncSetAttribute(batched_kernel<BT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(device_info().smem_optin - fa.sharedSizeBytes));
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(batched)");
        attr_done[dev] = true;
    }
    return CKM_OK;
}

template <int BT>
int launch_batched_t(const BatchJobDev* jobs, const BatchSegment* segs, uint32_t num_segs, unsigned int* work,
                     float tol, uint32_t max_it, uint32_t grid, uint32_t tile, uint32_t flush_tiles, size_t cent_cap,
                     size_t acc_cap, uint32_t use_umma, cudaStream_t s) {
    const size_t smem = cent_cap + acc_cap;
    int st = ensure_batched_attr<BT>();
    if (st) return st;
    if (grid == 0) return CKM_OK;
    cudaError_t e0 = cudaMemsetAsync(work, 0, sizeof(unsigned int), s);
    if (e0 != cudaSuccess) return cuda_fail(e0, "batched work counter");
    batched_kernel<BT><<<grid, BT, smem, s>>>(jobs, segs, num_segs, work, tol, max_it, tile, flush_tiles, cent_cap,
                                              acc_cap, use_umma);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "batched launch");
}

}  // namespace

int launch_batched(const BatchJobDev* jobs, const BatchSegment* segs, uint32_t num_segs, unsigned int* work,
                   float tol, uint32_t max_it, uint32_t grid, uint32_t block, uint32_t tile, uint32_t flush_tiles,
                   size_t cent_cap, size_t acc_cap, uint32_t use_umma, cudaStream_t s) {
    if (block == 512)
        return launch_batched_t<512>(jobs, segs, num_segs, work, tol, max_it, grid, tile, flush_tiles, cent_cap,
                                     acc_cap, use_umma, s);
    if (block != 256) return fail(CKM_ERR_INVALID_ARGUMENT, "batched: CTA size must be 256 or 512");
    return launch_batched_t<256>(jobs, segs, num_segs, work, tol, max_it, grid, tile, flush_tiles, cent_cap, acc_cap,
                                 use_umma, s);
}

int batched_blocks_per_sm(size_t smem, uint32_t block, int* out) {
    if (block != 256 && block != 512) return fail(CKM_ERR_INVALID_ARGUMENT, "batched: CTA size must be 256 or 512");
    int st = block == 512 ? ensure_batched_attr<512>() : ensure_batched_attr<256>();
    if (st) return st;
    const cudaError_t e =
        block == 512 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, batched_kernel<512>, 512, smem)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, batched_kernel<256>, 256, smem);
    return e == cudaSuccess ? CKM_OK : fail(CKM_ERR_CUDA, "occupancy(batched)");
}

}  // namespace ckm

namespace ckm {
namespace {

__global__ void batch_sync_kernel(const BatchJobDev* __restrict__ jobs, uint32_t num_jobs) {
    for (uint32_t j = blockIdx.x; j < num_jobs; j += gridDim.x) {
        const BatchJobDev J = jobs[j];
        if ((J.status->parity & 1u) == 0u) continue;
        const uint32_t kd = J.k * J.d;
        for (uint32_t i = threadIdx.x; i < kd; i += blockDim.x) J.cent[0][i] = J.cent[1][i];
        __syncthreads();
        if (threadIdx.x == 0) J.status->parity = 0u;
    }
}

}  // namespace

int launch_batch_sync(const BatchJobDev* jobs, uint32_t num_jobs, cudaStream_t s) {
    if (num_jobs == 0) return CKM_OK;
    const uint32_t grid = num_jobs < 4096u ? num_jobs : 4096u;
    batch_sync_kernel<<<grid, 256, 0, s>>>(jobs, num_jobs);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "batch sync launch");
}

}  // namespace ckm

// ----------------------------------------------------------------------------
// The fused functor's tensor-core route: one job on the batched kernel.
// ----------------------------------------------------------------------------
namespace ckm {
namespace {

// Layout of the scratch extension (FUSED_UMMA_EXT bytes): the job record,
// its status, tile ticket and work counter, then the segment list.
constexpr size_t FU_JOB = 0, FU_STATUS = 128, FU_TICKET = 144, FU_WORK = 148, FU_SEGS = 256;
constexpr uint32_t FU_MAX_SEGS = (uint32_t)((FUSED_UMMA_EXT - FU_SEGS) / sizeof(BatchSegment));
constexpr uint32_t FU_TILE = 4096;
// Where the route pays (measured per call against rows_kernel's TF32 mma.sync
// screen, 20 calls each): at n = 2^20 with k = 256 it takes 603 against 786 us
// (d = 64) and 344 against 391 us (d = 32); at k = 64 or n <= 2^18 rows_kernel
// is faster (a 4096-point tile per segment leaves most SMs idle on small n,
// and each segment restages the centroids).
constexpr uint64_t FU_MIN_POINTS = 1ull << 20;
constexpr uint32_t FU_MIN_K = 128;

__global__ void fused_umma_setup_kernel(unsigned char* ext, BatchJobDev job, uint32_t nsegs, uint32_t per) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *reinterpret_cast<BatchJobDev*>(ext + FU_JOB) = job;
        BatchStatus st;
        st.shift = 0.0f;
        st.iterations = 0u;
        st.parity = 0u;  // centroids in cent[0] (the old ones); the means go to cent[1]
        st.flags = 0u;
        *reinterpret_cast<BatchStatus*>(ext + FU_STATUS) = st;
        *reinterpret_cast<unsigned int*>(ext + FU_TICKET) = 0u;
        *reinterpret_cast<unsigned int*>(ext + FU_WORK) = 0u;
    }
    BatchSegment* segs = reinterpret_cast<BatchSegment*>(ext + FU_SEGS);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsegs; i += gridDim.x * blockDim.x) {
        BatchSegment sg;
        sg.job = 0u;
        sg.tile_begin = i * per;
        sg.tile_end = min((i + 1u) * per, job.num_tiles);
        sg.pad = 0u;
        segs[i] = sg;
    }
}

}  // namespace

int launch_fused_umma(const FusedF32& a, cudaStream_t s) {
    const char* env = std::getenv("CKM_FUSED_UMMA");  // tuning: "0" never, "1" at any n
    const bool never = env && env[0] == '0', always = env && env[0] == '1';
    const DeviceInfo& di = device_info();
    if (never || a.mode != CKM_MODE_FINALIZE || !a.scratch.ext || di.cc_major != 10 || (a.d != 32 && a.d != 64) ||
        a.k < UMMA_MIN_K || a.k > UMMA_MAX_K || a.n == 0 || (!always && (a.n < FU_MIN_POINTS || a.k < FU_MIN_K)))
        return -1000;
    const uint64_t num_tiles = (a.n + FU_TILE - 1) / FU_TILE;
    if (num_tiles > 0xffffffffull) return -1000;
    const uint32_t per = (uint32_t)((num_tiles + FU_MAX_SEGS - 1) / FU_MAX_SEGS);
    const uint32_t nsegs = (uint32_t)((num_tiles + per - 1) / per);
    // shared-memory caps as the batch schedule sets them for a tensor-core job
    const size_t need_c = ((size_t)a.k * a.d + ((a.k + 3u) & ~3u)) * sizeof(float);
    const size_t budget = std::min<size_t>(di.smem_optin - 1024, 200 * 1024);
    const size_t cent_cap = std::min((need_c + 255) & ~size_t(255), budget / 2);
    const size_t acc_cap = budget - cent_cap;
    unsigned char* ext = a.scratch.ext;
    BatchJobDev job;
    std::memset(&job, 0, sizeof(job));
    job.points = a.points;
    job.cent[0] = const_cast<float*>(a.centroids);  // read only: the kernel writes cent[parity ^ 1]
    job.cent[1] = a.new_centroids;
    job.labels = a.labels;
    job.masses = a.masses;
    job.sums = a.scratch.sums;
    job.msum = a.scratch.masses;
    job.ticket = reinterpret_cast<unsigned int*>(ext + FU_TICKET);
    job.status = reinterpret_cast<BatchStatus*>(ext + FU_STATUS);
    job.n = a.n;
    job.d = a.d;
    job.k = a.k;
    job.num_tiles = (uint32_t)num_tiles;
    fused_umma_setup_kernel<<<1, 256, 0, s>>>(ext, job, nsegs, per);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "fused tensor-core setup launch");
    const uint32_t grid = std::min<uint32_t>((uint32_t)di.sm_count, nsegs);
    return launch_batched(reinterpret_cast<const BatchJobDev*>(ext + FU_JOB),
                          reinterpret_cast<const BatchSegment*>(ext + FU_SEGS), nsegs,
                          reinterpret_cast<unsigned int*>(ext + FU_WORK), 0.0f, 0u, grid, 512, FU_TILE, 16, cent_cap,
                          acc_cap, 1u, s);
}

}  // namespace ckm
