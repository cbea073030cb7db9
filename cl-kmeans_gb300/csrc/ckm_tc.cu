// Tensor-core Lloyd iteration for large k*d (tcgen05, sm_100 family).
//
// The labeling step of the reference (kmeans_naive.cpp:48-63: for every
// point, the cluster with the smallest FP32 distance sum_f (x_f - c_f)^2,
// strict '<' from cluster 0, so the lowest index wins a tie and NaN never
// wins) is computed as a GEMM of scores
//     score(x, c) = |c|^2 - 2 x.c        (argmin over c = argmin of |x - c|^2)
// on fp16 operands with f32 accumulation in tensor memory, and certified:
//
//   - points and centroids are scaled by powers of two (sx, sc) so that every
//     coordinate fits fp16 (|.| <= 2^15) and rounded to fp16 once;
//   - a rigorous bound T(x) covers the fp16 rounding of both operands (by the
//     norms of the actual rounding errors, measured when the operands are
//     made, through Cauchy-Schwarz), the f32 accumulation (one ulp per
//     addition), the rounding of |c|^2 and of the score itself, the FP32
//     rounding of the reference distance ((d + 2) 2^-24 relative) and FP32
//     underflow (2^-150 absolute per operation).  A cluster whose score is more than T above the best score
//     cannot reach or tie the reference's minimum, so the reference's label
//     is among the clusters within T of the best (the candidates);
//   - one candidate: that is the label.  2..CAP candidates: the kernel
//     computes their distances with the reference arithmetic (t = x_f - c_f,
//     acc = fma(t, t, acc), f ascending) and keeps the smallest, lowest index
//     on a tie.  More: the point goes to tc_recheck_kernel (all clusters,
//     exact arithmetic).
//
// The centroid update (kmeans_naive.cpp:65-83: per-cluster sums of the
// points, divided by the counts) runs after labeling as a counting sort of the
// points by label and a segmented sum over an FP32 row-major copy of the
// points, accumulated as an unevaluated pair of floats and merged in FP64.
//
// Kernels per iteration: centroid statistics, centroid packing, labeling
// (persistent, warp-specialised: TMA producer warp, MMA warp, two epilogue
// warpgroups over double-buffered tensor memory), exact recheck, offsets,
// scatter, segmented sums, finalisation.
#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "ckm_device.cuh"
#include "ckm_internal.h"
#include "ckm_tc.h"
#include "ckm_umma.cuh"

namespace ckm {
namespace {

constexpr int TILE_M = 128;          // points per tile (tensor-memory lanes)
constexpr int PAIR_M = 2 * TILE_M;   // a pair of tiles shares each centroid chunk
constexpr int EPI_WARPS = 8;         // two warpgroups, one per tile of a pair
constexpr int EPI_THREADS = EPI_WARPS * 32;
constexpr int PRODUCER_WARP = 8;
constexpr int MMA_WARP = 9;
constexpr int LABEL_THREADS = 320;
constexpr int CAP = 8;               // candidates kept per point in the label kernel
constexpr int GRP = 16;              // scores per warp-uniform append test
constexpr uint32_t CN_SMEM_MAX = 2048;  // |c|^2 of up to this many clusters is kept in shared memory
constexpr int MAX_A_STAGES = 2;
constexpr int MAX_B_STAGES = 4;
constexpr unsigned long long WAIT_NS = 2000000000ull;  // bounded waits give up after 2 s
constexpr uint32_t NONE = 0xffffffffu;

// Power-of-two exponent e such that 2^e * maxabs <= 2^15 (fp16 safe), kept in
// [-60, 60] so that products of two scales and their inverses stay normal.
__host__ __device__ inline int scale_exponent(float maxabs) {
    if (!(maxabs > 0.0f) || isinf(maxabs)) return 0;
    int e = 0;
    frexpf(maxabs, &e);  // maxabs = m 2^e, m in [0.5, 1): maxabs <= 2^e
    int s = 15 - e;
    return s < -60 ? -60 : (s > 60 ? 60 : s);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// try_wait with a suspend-time hint: a thread whose phase is not complete
// sleeps (up to hint_ns, or until the phase completes) instead of spinning,
// so waiting warps take no issue slots from the warps doing the work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity, uint32_t hint_ns) {
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

// mbarrier wait with a time limit and a shared abort flag: returns false when
// another role aborted or the phase did not complete within WAIT_NS.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity, volatile unsigned int* abort_flag) {
    if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
        if (*abort_flag) return false;
        if (global_ns() - t0 > WAIT_NS) {
            *abort_flag = 1u;
            return false;
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// counts[c] += 1 for every calling thread, with one atomic per distinct c
// among the calling threads of a warp.  In a cluster-ordered point set the
// points of a warp, and those that all SMs label at the same time, mostly
// share one or two labels: one atomic per point would serialise at those
// few counters.
__device__ __forceinline__ void count_label(uint32_t* counts, uint32_t c) {
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    const cg::coalesced_group same = cg::labeled_partition(g, c);
    if (same.thread_rank() == 0) atomicAdd(&counts[c], same.size());
}

// Instruction descriptor, kind::f16: D f32, A and B both fp16 or both bf16
// (operand format 0 or 1 in the A and B format fields), both K-major.
__host__ __device__ __forceinline__ uint32_t idesc_f16_f32(uint32_t M, uint32_t N, uint32_t precision = 0) {
    const uint32_t ab = precision == CKM_TC_BF16 ? (1u << 7) | (1u << 10) : 0u;
    return (1u << 4) | ab | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// One operand value rounded to the point set's 2-byte type (fp16 or bf16):
// the stored bits and the rounded value back in FP32.
__device__ __forceinline__ uint16_t round_operand(float v, uint32_t precision, float& back) {
    if (precision == CKM_TC_BF16) {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        back = __bfloat162float(h);
        return *reinterpret_cast<const uint16_t*>(&h);
    }
    const __half h = __float2half_rn(v);
    back = __half2float(h);
    return *reinterpret_cast<const uint16_t*>(&h);
}

// 32 consecutive accumulator columns of this thread's TMEM lane (no wait).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32], int base) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr + (uint32_t)base));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// --------------------------------------------------------------------------
// Point preparation (once per point set)
// --------------------------------------------------------------------------

// max |x_f| over the finite coordinates (NaN is skipped by fmaxf).
__global__ void __launch_bounds__(256) tc_points_maxabs_kernel(const float* __restrict__ P, uint64_t total,
                                                               TcPointsHeader* hdr) {
    float m = 0.0f;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const float a = fabsf(P[i]);
        if (!isinf(a)) m = fmaxf(m, a);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(&hdr->maxabs_bits, __float_as_uint(m));
}

// 32 points per CTA: the column-major coordinates are staged in shared
// memory, then each warp writes whole rows: the scaled fp16 row (zero padded
// to d_pad), the FP32 row (zero padded to d4) and an upper bound of |x|.
__global__ void __launch_bounds__(256) tc_points_convert_kernel(const float* __restrict__ P, uint64_t n, uint32_t d,
                                                                uint32_t d_pad, uint32_t d4,
                                                                const TcPointsHeader* __restrict__ hdr,
                                                                uint16_t* __restrict__ ph, float* __restrict__ norms,
                                                                float* __restrict__ errn, float* __restrict__ prm,
                                                                uint32_t* __restrict__ orig) {
    extern __shared__ float s_tile[];  // [d][33]
    const float sx = ldexpf(1.0f, scale_exponent(__uint_as_float(hdr->maxabs_bits)));
    const uint32_t prec = hdr->precision;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t p0 = (uint64_t)blockIdx.x * 32; p0 < n; p0 += (uint64_t)gridDim.x * 32) {
        const uint64_t p = p0 + lane;
        for (uint32_t f = warp; f < d; f += 8) s_tile[f * 33 + lane] = p < n ? P[(uint64_t)f * n + p] : 0.0f;
        __syncthreads();
        for (int r = warp; r < 32; r += 8) {
            const uint64_t q = p0 + r;
            if (q >= n) break;
            float ss = 0.0f, ee = 0.0f;
            for (uint32_t f = lane; f < d_pad; f += 32) {
                const float v = f < d ? s_tile[f * 33 + r] : 0.0f;
                ss = fmaf(v, v, ss);
                float back;
                ph[q * d_pad + f] = round_operand(v * sx, prec, back);
                const float e = back - v * sx;  // exact: both within a factor 2 (or e = -v sx)
                ee = fmaf(e, e, ee);
            }
            for (uint32_t f = lane; f < d4; f += 32) prm[q * d4 + f] = f < d ? s_tile[f * 33 + r] : 0.0f;
            for (int o = 16; o > 0; o >>= 1) {
                ss += __shfl_xor_sync(0xffffffffu, ss, o);
                ee += __shfl_xor_sync(0xffffffffu, ee, o);
            }
            // FP32 sum of d + 5 non-negative terms: relative error below
            // (d + 5) 2^-24 < 2^-14; the square root adds half an ulp
            if (lane == 0) {
                norms[q] = sqrtf(ss * (1.0f + 0x1p-14f)) * (1.0f + 0x1p-20f);
                // + d 2^-149: v sx may have been rounded where it fell below
                // FP32's normal range
                errn[q] = (sqrtf(ee * (1.0f + 0x1p-14f)) * (1.0f + 0x1p-20f) + (float)d * 0x1p-149f) / sx;
                orig[q] = (uint32_t)q;
            }
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// Centroid preparation (every iteration)
// --------------------------------------------------------------------------

// Per centroid: validity (all coordinates finite; an empty cluster of the
// previous iteration is NaN and never wins, as in the reference), |c|^2 in
// FP64 rounded to FP32 (+inf for invalid and padding rows), the FP32
// row-major copy used by the exact distance, max |c_f| and an upper bound of
// |c| over the valid rows.
__global__ void tc_centroid_stats_kernel(const float* __restrict__ C, uint32_t k, uint32_t d, uint32_t k_pad,
                                         uint32_t d4, float* __restrict__ cent_rm, float* __restrict__ cn2,
                                         TcIterDev* it) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < k_pad; c += gridDim.x * blockDim.x) {
        if (c >= k) {
            cn2[c] = __int_as_float(0x7f800000);
            continue;
        }
        bool valid = true;
        double s = 0.0;
        float amax = 0.0f;
        float* row = cent_rm + (uint64_t)c * d4;
        for (uint32_t f = 0; f < d; ++f) {
            const float v = C[(uint64_t)f * k + c];
            if (!isfinite(v)) valid = false;
            s = fma((double)v, (double)v, s);
            amax = fmaxf(amax, fabsf(v));
            row[f] = v;
        }
        for (uint32_t f = d; f < d4; ++f) row[f] = 0.0f;
        cn2[c] = valid ? (float)s : __int_as_float(0x7f800000);
        if (valid) {
            atomicMax(&it->cmax_bits, __float_as_uint(__double2float_ru(sqrt(s) * (1.0 + 0x1p-40))));
            atomicMax(&it->cabs_bits, __float_as_uint(amax));
        }
    }
}

// Centroids scaled by sc in the point set's operand type (fp16 or bf16),
// K-major [k_pad][d_pad] (invalid and padding rows zero), and a bound of the
// rounding error of the valid rows.
__global__ void tc_centroid_pack_kernel(const float* __restrict__ C, uint32_t k, uint32_t d, uint32_t k_pad,
                                        uint32_t d_pad, const float* __restrict__ cn2, uint16_t* __restrict__ ch,
                                        const TcPointsHeader* __restrict__ hdr, TcIterDev* it) {
    const int ec = scale_exponent(__uint_as_float(it->cabs_bits));
    const float sc = ldexpf(1.0f, ec);
    const uint32_t prec = hdr->precision;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < k_pad; c += gridDim.x * blockDim.x) {
        const bool valid = c < k && cn2[c] < __int_as_float(0x7f800000);
        uint16_t* row = ch + (uint64_t)c * d_pad;
        double ee = 0.0;
        for (uint32_t f = 0; f < d_pad; ++f) {
            const float b = (valid && f < d) ? C[(uint64_t)f * k + c] * sc : 0.0f;
            float back;
            row[f] = round_operand(b, prec, back);
            const double e = (double)back - (double)b;
            ee = fma(e, e, ee);
        }
        if (valid)
            atomicMax(&it->fmax_bits,
                      __float_as_uint(__double2float_ru((sqrt(ee) * (1.0 + 0x1p-40) + d * 0x1p-149) / sc)));
    }
}

// The per-iteration scale and certificate constants (one thread).  With x
// the point, e its fp16 rounding error (both unscaled), cm >= max |c| and
// fm >= max |fp16 error of c| over valid centroids, g = 2 d_pad 2^-23 (f32
// accumulation, one ulp per addition) and rho = (d + 2) 2^-24 (the
// reference's FP32 distance):
//   |score error| <= 2 (|x| fm + |e| (cm + fm) + g (|x| + |e|)(cm + fm))
//                    + 2^-23 (|x| + cm)^2       (|c|^2 and the score rounded)
//   T = 2 |score error| + 2 rho (|x| + cm)^2 + (d + 8) 2^-146 (underflow)
// (Cauchy-Schwarz on the exact rounding errors: |sum e_f c_f| <= |e||c|.)
__global__ void tc_params_kernel(uint32_t d, uint32_t d_pad, const TcPointsHeader* __restrict__ hdr, TcIterDev* it) {
    const int ex = scale_exponent(__uint_as_float(hdr->maxabs_bits));
    const int ec = scale_exponent(__uint_as_float(it->cabs_bits));
    const double sx = ldexp(1.0, ex), scd = ldexp(1.0, ec);
    const double cm = (double)__uint_as_float(it->cmax_bits), fm = (double)__uint_as_float(it->fmax_bits);
    const double gam = 2.0 * d_pad * 0x1p-23, safety = 1.0 + 0x1p-10;
    it->alpha = (float)(-2.0 / (sx * scd));  // a power of two: exact
    it->t1 = __double2float_ru((4.0 * fm + 4.0 * gam * (cm + fm)) * safety);
    it->te = __double2float_ru((4.0 * (cm + fm) + 4.0 * gam * (cm + fm)) * safety);
    it->t2 = __double2float_ru((2.0 * 0x1p-23 * 1.01 + 2.0 * (d + 2.0) * 0x1p-24 * 1.01) * safety);
    it->t0 = __double2float_ru((d + 8.0) * 0x1p-146);
    it->cm = __double2float_ru(cm);
}

// --------------------------------------------------------------------------
// Labeling kernel
// --------------------------------------------------------------------------
struct LabelParams {
    const float* norms;          // upper bound of |x| per point
    const float* errn;           // upper bound of |fp16(x sx) / sx - x| per point
    const float* x_rm;           // FP32 points, row-major [n][d4]
    const uint32_t* orig;        // caller's index of each point of the set
    const uint32_t* precision;   // the point set's operand type (its header)
    const float* c_rm;           // FP32 centroids, row-major [k][d4]
    const float* cn2;            // |c|^2 [k_pad]
    TcIterDev* it;
    uint32_t* labels;            // caller's order
    uint32_t* slabels;           // the set's order (on entry: the previous call's, read for the chunk order)
    uint32_t* counts;            // points per label in this call
    uint32_t* flagged;           // points for the full recheck
    uint32_t* res_pts;           // points with 2+ candidates (tc_resolve_kernel)
    uint32_t* res_cands;         // their candidates, CAP per point, NONE-padded
    uint64_t n;
    uint32_t d, d4, d_pad, k, chunks, num_pairs, a_stages, b_stages;
};

// First chunk of pair q: the chunk holding the previous label of the pair's
// middle point.  In a cluster-ordered set most points of the pair share that
// label, so the running minimum is (nearly) final after the first chunk and
// later chunks append only true candidates.  Any value gives a valid order
// (the chunks are visited cyclically from it), so an uninitialised or stale
// label only costs time.  The label is read before this call writes it: the
// pair's epilogue writes its labels after all three roles have read it.
template <int BN>
__device__ __forceinline__ uint32_t home_chunk(const LabelParams& prm, uint32_t q) {
    uint64_t pm = (uint64_t)q * PAIR_M + TILE_M;
    if (pm >= prm.n) pm = (uint64_t)q * PAIR_M;
    const uint32_t lab = *(volatile const uint32_t*)(prm.slabels + pm);
    return lab < prm.k ? (lab / BN) % prm.chunks : 0u;
}

// One CTA per SM, looping over pairs of 128-point tiles.  Warp 8 (one lane)
// streams the pair's fp16 rows and the centroid chunks by TMA; warp 9 (one
// lane) issues the MMAs of each chunk for both tiles into tensor memory
// (two buffers per tile); warps 0-3 score tile 0 and warps 4-7 tile 1, one
// point per thread (= one TMEM lane).  Per chunk a thread loads its BN
// scores, hands the buffer back, takes the chunk minimum into its running
// minimum m and appends every cluster whose score is within T of m to its
// candidate list in shared memory; entries that fall out of range when m
// drops later are filtered at the end.
template <int BN, bool CN_SMEM>
__global__ void __launch_bounds__(LABEL_THREADS, 1)
    tc_label_kernel(const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b,
                    const LabelParams prm) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar_af[MAX_A_STAGES], bar_ae[MAX_A_STAGES];
    __shared__ __align__(8) uint64_t bar_bf[MAX_B_STAGES], bar_be[MAX_B_STAGES];
    __shared__ __align__(8) uint64_t bar_tf[4], bar_te[4], bar_fin;
    __shared__ uint32_t s_tmem;
    __shared__ unsigned int s_abort;
    volatile unsigned int* abort_flag = &s_abort;

    const uint32_t raw = umma::smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const uint32_t a_bytes = PAIR_M * prm.d_pad * 2u, b_bytes = BN * prm.d_pad * 2u;
    const uint32_t sA = base, sB = base + prm.a_stages * a_bytes;
    float2* lists = reinterpret_cast<float2*>(smem_raw + (base - raw) + prm.a_stages * a_bytes + prm.b_stages * b_bytes);
    // |c|^2 of all clusters in shared memory when it fits (CN_SMEM)
    float* s_cn = reinterpret_cast<float*>(lists + (CAP + 1) * EPI_THREADS);
    if (CN_SMEM)
        for (uint32_t i = threadIdx.x; i < prm.chunks * BN; i += blockDim.x) s_cn[i] = __ldg(prm.cn2 + i);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t kblocks = prm.d_pad / 64u;

    if (threadIdx.x == 0) {
        for (uint32_t i = 0; i < prm.a_stages; ++i) {
            umma::mbar_init(umma::smem_u32(&bar_af[i]), 1);
            umma::mbar_init(umma::smem_u32(&bar_ae[i]), 1);
        }
        for (uint32_t i = 0; i < prm.b_stages; ++i) {
            umma::mbar_init(umma::smem_u32(&bar_bf[i]), 1);
            umma::mbar_init(umma::smem_u32(&bar_be[i]), 1);
        }
        for (int i = 0; i < 4; ++i) {
            umma::mbar_init(umma::smem_u32(&bar_tf[i]), 1);
            umma::mbar_init(umma::smem_u32(&bar_te[i]), 4);  // the four warps of a warpgroup
        }
        umma::mbar_init(umma::smem_u32(&bar_fin), 1);
        umma::mbar_fence_init();
        s_abort = 0u;
    }
    if (warp == MMA_WARP) umma::tmem_alloc(umma::smem_u32(&s_tmem), 4 * BN);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = s_tmem;

    if (warp == PRODUCER_WARP) {
        if (lane == 0) {
            uint32_t ia = 0, ib = 0;  // loads issued so far (A pairs, B chunks)
            bool ok = true;
            for (uint32_t q = blockIdx.x; ok && q < prm.num_pairs; q += gridDim.x) {
                const uint32_t sa = ia % prm.a_stages, pa = (ia / prm.a_stages) & 1u;
                if (!(ok = wait_phase(umma::smem_u32(&bar_ae[sa]), pa ^ 1u, abort_flag))) break;
                umma::mbar_arrive_expect_tx(umma::smem_u32(&bar_af[sa]), a_bytes);
                for (uint32_t kb = 0; kb < kblocks; ++kb)
                    umma::tma_load_2d(sA + sa * a_bytes + kb * (PAIR_M * 128u), &tm_a, (int)(kb * 64),
                                      (int)(q * PAIR_M), umma::smem_u32(&bar_af[sa]));
                ++ia;
                const uint32_t j0 = home_chunk<BN>(prm, q);
                for (uint32_t j = 0; j < prm.chunks; ++j) {
                    const uint32_t jj = j0 + j < prm.chunks ? j0 + j : j0 + j - prm.chunks;
                    const uint32_t sb = ib % prm.b_stages, pb = (ib / prm.b_stages) & 1u;
                    if (!(ok = wait_phase(umma::smem_u32(&bar_be[sb]), pb ^ 1u, abort_flag))) break;
                    umma::mbar_arrive_expect_tx(umma::smem_u32(&bar_bf[sb]), b_bytes);
                    for (uint32_t kb = 0; kb < kblocks; ++kb)
                        umma::tma_load_2d(sB + sb * b_bytes + kb * (BN * 128u), &tm_b, (int)(kb * 64), (int)(jj * BN),
                                          umma::smem_u32(&bar_bf[sb]));
                    ++ib;
                }
            }
            if (!ok) {
                // another role gave up: let the copies already issued land
                // (bounded) before the CTA exits
                for (uint32_t i = 0; i < prm.a_stages; ++i) {
                    const uint32_t issued = ia > i ? (ia - i + prm.a_stages - 1) / prm.a_stages : 0u;
                    if (issued) umma::mbar_wait(umma::smem_u32(&bar_af[i]), (issued - 1) & 1u, 1u << 20);
                }
                for (uint32_t i = 0; i < prm.b_stages; ++i) {
                    const uint32_t issued = ib > i ? (ib - i + prm.b_stages - 1) / prm.b_stages : 0u;
                    if (issued) umma::mbar_wait(umma::smem_u32(&bar_bf[i]), (issued - 1) & 1u, 1u << 20);
                }
            }
        }
    } else if (warp == MMA_WARP) {
        if (lane == 0) {
            const uint32_t idesc = idesc_f16_f32(TILE_M, BN, *prm.precision);
            uint32_t ia = 0, ib = 0, ic = 0;
            bool ok = true;
            for (uint32_t q = blockIdx.x; ok && q < prm.num_pairs; q += gridDim.x, ++ia) {
                const uint32_t sa = ia % prm.a_stages, pa = (ia / prm.a_stages) & 1u;
                if (!(ok = wait_phase(umma::smem_u32(&bar_af[sa]), pa, abort_flag))) break;
                for (uint32_t j = 0; ok && j < prm.chunks; ++j, ++ib, ++ic) {
                    const uint32_t sb = ib % prm.b_stages, pb = (ib / prm.b_stages) & 1u;
                    if (!(ok = wait_phase(umma::smem_u32(&bar_bf[sb]), pb, abort_flag))) break;
                    const uint32_t buf = ic & 1u, pt = (ic >> 1) & 1u;
                    for (uint32_t u = 0; u < 2; ++u) {
                        if (!(ok = wait_phase(umma::smem_u32(&bar_te[u * 2 + buf]), pt ^ 1u, abort_flag))) break;
                        umma::fence_after_sync();
                        const uint32_t dt = tmem + (u * 2 + buf) * BN;
                        for (uint32_t ks = 0; ks < prm.d_pad / 16u; ++ks) {
                            const uint32_t kb = ks >> 2, sub = ks & 3u;
                            const uint64_t ad =
                                umma::sw128_desc(sA + sa * a_bytes + kb * (PAIR_M * 128u) + u * (TILE_M * 128u) + sub * 32u);
                            const uint64_t bd = umma::sw128_desc(sB + sb * b_bytes + kb * (BN * 128u) + sub * 32u);
                            umma::mma_bf16(dt, ad, bd, idesc, ks > 0 ? 1u : 0u);
                        }
                        umma::mma_commit(umma::smem_u32(&bar_tf[u * 2 + buf]));
                    }
                    umma::mma_commit(umma::smem_u32(&bar_be[sb]));
                }
                umma::mma_commit(umma::smem_u32(&bar_ae[sa]));
            }
            // every MMA issued has completed before tensor memory is freed
            umma::mma_commit(umma::smem_u32(&bar_fin));
            umma::mbar_wait(umma::smem_u32(&bar_fin), 0u, 1u << 22);
        }
    } else {
        // ---- epilogue: warps 0-7 ----
        const uint32_t u = (uint32_t)warp >> 2, lg = (uint32_t)warp & 3u;
        const uint32_t row = lg * 32u + (uint32_t)lane;
        const uint32_t etid = threadIdx.x;
        const float alpha = prm.it->alpha, t0 = prm.it->t0, t1 = prm.it->t1, te = prm.it->te, t2 = prm.it->t2,
                    cm = prm.it->cm;
        const float2 al2 = make_float2(alpha, alpha);
        const float INF = __int_as_float(0x7f800000);
        const uint32_t lane_addr = tmem + ((lg * 32u) << 16);
        uint32_t ic = 0;
        bool aborted = false;
        for (uint32_t q = blockIdx.x; !aborted && q < prm.num_pairs; q += gridDim.x) {
            const uint64_t p = (uint64_t)q * PAIR_M + u * TILE_M + row;
            const bool valid = p < prm.n;
            const float xn = valid ? __ldg(prm.norms + p) : 0.0f;
            const float xe = valid ? __ldg(prm.errn + p) : 0.0f;
            const float T = fmaf(t2 * (xn + cm), xn + cm, fmaf(te, xe, fmaf(t1, xn, t0))) * (1.0f + 0x1p-10f);
            float m = INF;
            uint32_t cnt = 0;
            bool ovf = false;
            const uint32_t j0 = home_chunk<BN>(prm, q);
            for (uint32_t j = 0; j < prm.chunks; ++j, ++ic) {
                const uint32_t jj = j0 + j < prm.chunks ? j0 + j : j0 + j - prm.chunks;
                const uint32_t buf = ic & 1u, pt = (ic >> 1) & 1u;
                int ok = 1;
                if (lane == 0) ok = wait_phase(umma::smem_u32(&bar_tf[u * 2 + buf]), pt, abort_flag);
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    aborted = true;
                    break;
                }
                umma::fence_after_sync();
                uint32_t r[BN];
#pragma unroll
                for (int i = 0; i < BN / 32; ++i)
                    tmem_ld32_nowait(lane_addr + (u * 2 + buf) * BN, *reinterpret_cast<uint32_t(*)[32]>(&r[32 * i]),
                                     32 * i);
                tmem_wait_ld();
                umma::fence_before_sync();
                __syncwarp();
                if (lane == 0) mbar_arrive(umma::smem_u32(&bar_te[u * 2 + buf]));

                float s[BN];
                const float4* cn4 = reinterpret_cast<const float4*>((CN_SMEM ? s_cn : prm.cn2) + (uint64_t)jj * BN);
#pragma unroll
                for (int i = 0; i < BN / 4; ++i) {
                    const float4 c = CN_SMEM ? cn4[i] : __ldg(cn4 + i);
                    const float2 a = fma2(make_float2(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1])), al2,
                                          make_float2(c.x, c.y));
                    const float2 b = fma2(make_float2(__uint_as_float(r[4 * i + 2]), __uint_as_float(r[4 * i + 3])),
                                          al2, make_float2(c.z, c.w));
                    s[4 * i] = a.x;
                    s[4 * i + 1] = a.y;
                    s[4 * i + 2] = b.x;
                    s[4 * i + 3] = b.y;
                }
                // minima of groups of 16 scores, then of the chunk
                float gm[BN / GRP];
#pragma unroll
                for (int g = 0; g < BN / GRP; ++g) {
                    const float* t = &s[g * GRP];
                    const float a = fmin3(t[0], t[1], t[2]), b = fmin3(t[3], t[4], t[5]),
                                c = fmin3(t[6], t[7], t[8]), e = fmin3(t[9], t[10], t[11]),
                                f = fmin3(t[12], t[13], t[14]);
                    gm[g] = fminf(fmin3(a, b, c), fmin3(e, f, t[15]));
                }
                float mn = gm[0];
#pragma unroll
                for (int g = 1; g < BN / GRP; ++g) mn = fminf(mn, gm[g]);
                m = fminf(m, mn);
                const float cut = m + T;
                // appends: a group is scanned only when one of the warp's points
                // has a score in range there (a warp-uniform branch)
                const uint32_t cbase = jj * BN;
#pragma unroll
                for (int g = 0; g < BN / GRP; ++g) {
                    if (__any_sync(0xffffffffu, valid && gm[g] <= cut)) {
#pragma unroll
                        for (int i = 0; i < GRP; ++i) {
                            const float v = s[g * GRP + i];
                            if (valid && v <= cut) {
                                lists[(cnt < CAP ? cnt : CAP) * EPI_THREADS + etid] =
                                    make_float2(v, __uint_as_float(cbase + g * GRP + i));
                                ++cnt;
                            }
                        }
                    }
                }
                if (cnt > CAP) {
                    ovf = true;  // entries were lost: the point goes to the full recheck
                    cnt = CAP;
                } else if (cnt >= CAP / 2) {
                    uint32_t w = 0;  // drop entries that are out of range now
                    for (uint32_t e = 0; e < cnt; ++e) {
                        const float2 v = lists[e * EPI_THREADS + etid];
                        if (v.x <= cut) lists[(w++) * EPI_THREADS + etid] = v;
                    }
                    cnt = w;
                }
            }
            if (aborted) break;

            // ---- resolution ----
            // Filter the list with the final m.  One candidate: the label.  Two
            // or more: a record (point, candidates) for tc_resolve_kernel.
            // Overflow or no finite score: the full exact recheck.
            const float cut = m + T;
            bool flag = valid && (ovf || !(m > -INF && m < INF));
            uint32_t label = NONE, nc = 0;
            if (valid && !flag) {
                for (uint32_t e = 0; e < cnt; ++e) {
                    const float2 v = lists[e * EPI_THREADS + etid];
                    const uint32_t c = __float_as_uint(v.y);
                    if (v.x <= cut && c < prm.k) {
                        lists[nc * EPI_THREADS + etid].y = v.y;  // compact the candidates to the front
                        ++nc;
                        label = c;
                    }
                }
                if (nc == 0) flag = true;
            }
            const bool need = valid && !flag && nc >= 2;
            const unsigned int needm = __ballot_sync(0xffffffffu, need);
            uint32_t slot0 = 0;
            if (lane == 0 && needm) slot0 = atomicAdd(&prm.it->resolved, (unsigned)__popc(needm));
            slot0 = __shfl_sync(0xffffffffu, slot0, 0);
            if (need) {
                const uint32_t slot = slot0 + __popc(needm & ((1u << lane) - 1u));
                prm.res_pts[slot] = (uint32_t)p;
                uint32_t* rc = prm.res_cands + (uint64_t)slot * CAP;
                for (uint32_t e = 0; e < CAP; ++e)
                    rc[e] = e < nc ? __float_as_uint(lists[e * EPI_THREADS + etid].y) : NONE;
            } else if (valid) {
                if (flag) {
                    const unsigned int slot = atomicAdd(&prm.it->nflagged, 1u);
                    prm.flagged[slot] = (uint32_t)p;
                } else {
                    prm.labels[__ldg(prm.orig + p)] = label;
                    prm.slabels[p] = label;
                    count_label(prm.counts, label);
                }
            }
            const unsigned int novf = __popc(__ballot_sync(0xffffffffu, valid && ovf));
            if (lane == 0 && novf) atomicAdd(&prm.it->overflowed, novf);
        }
    }

    umma::fence_before_sync();
    __syncthreads();
    if (warp == MMA_WARP) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(tmem, 4 * BN);
    }
    if (threadIdx.x == 0 && s_abort) atomicExch(&prm.it->error, 1u);
}

// --------------------------------------------------------------------------
// Exact resolution of points with 2..CAP candidates: the reference distance
// (t = x_f - c_f, acc = fma(t, t, acc), f ascending) of every candidate, in
// one pass over the point's row; the smallest distance below FLT_MAX wins,
// the lowest index on a tie (= strict '<' in ascending cluster order,
// kmeans_naive.cpp:58-61).  Nothing below FLT_MAX: the full recheck.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) tc_resolve_kernel(const float* __restrict__ x_rm, const float* __restrict__ c_rm,
                                                         uint32_t d, uint32_t d4, const uint32_t* __restrict__ res_pts,
                                                         const uint32_t* __restrict__ res_cands,
                                                         const uint32_t* __restrict__ orig, TcIterDev* it,
                                                         uint32_t* __restrict__ flagged, uint32_t* __restrict__ labels,
                                                         uint32_t* __restrict__ slabels, uint32_t* __restrict__ counts) {
    const unsigned int count = it->resolved;
    for (unsigned int r = blockIdx.x * blockDim.x + threadIdx.x; r < count; r += gridDim.x * blockDim.x) {
        const uint32_t p = __ldg(res_pts + r);
        uint32_t cand[CAP];
        int nc = 0;
#pragma unroll
        for (int j = 0; j < CAP; ++j) {
            cand[j] = __ldg(res_cands + (uint64_t)r * CAP + j);
            nc += cand[j] != NONE;
        }
        float acc[CAP];
#pragma unroll
        for (int j = 0; j < CAP; ++j) acc[j] = 0.0f;
        const float4* xr = reinterpret_cast<const float4*>(x_rm + (uint64_t)p * d4);
        uint32_t f = 0;
        for (; f + 4 <= d; f += 4) {
            const float4 x = __ldg(xr + f / 4);
#pragma unroll
            for (int j = 0; j < CAP; ++j) {
                if (j < nc) {
                    const float4 c = __ldg(reinterpret_cast<const float4*>(c_rm + (uint64_t)cand[j] * d4) + f / 4);
                    float t = x.x - c.x;
                    acc[j] = fmaf(t, t, acc[j]);
                    t = x.y - c.y;
                    acc[j] = fmaf(t, t, acc[j]);
                    t = x.z - c.z;
                    acc[j] = fmaf(t, t, acc[j]);
                    t = x.w - c.w;
                    acc[j] = fmaf(t, t, acc[j]);
                }
            }
        }
        for (; f < d; ++f) {
            const float x = __ldg(x_rm + (uint64_t)p * d4 + f);
#pragma unroll
            for (int j = 0; j < CAP; ++j)
                if (j < nc) {
                    const float t = x - __ldg(c_rm + (uint64_t)cand[j] * d4 + f);
                    acc[j] = fmaf(t, t, acc[j]);
                }
        }
        float best = FLT_MAX;
        uint32_t bi = NONE;
#pragma unroll
        for (int j = 0; j < CAP; ++j)
            if (j < nc && (acc[j] < best || (acc[j] == best && bi != NONE && cand[j] < bi))) {
                best = acc[j];
                bi = cand[j];
            }
        if (bi == NONE) {
            const unsigned int slot = atomicAdd(&it->nflagged, 1u);
            flagged[slot] = p;
        } else {
            labels[__ldg(orig + p)] = bi;
            slabels[p] = bi;
            count_label(counts, bi);
        }
    }
}

// --------------------------------------------------------------------------
// Exact recheck of flagged points: the reference arithmetic over all
// clusters (t = x_f - c_f, acc = fma(t, t, acc) for f ascending; strict '<'
// from FLT_MAX; lowest index among equal minima; NaN never wins; label 0 when
// nothing is below FLT_MAX).  RECHECK_PTS points per CTA share every read of
// a centroid coordinate; each thread scans clusters tid, tid + 256, ...
// (ascending, so its own strict '<' keeps the lowest index) and the CTA
// merges the per-thread winners lexicographically.
// --------------------------------------------------------------------------
constexpr int RECHECK_PTS = 16;
__global__ void __launch_bounds__(256) tc_recheck_kernel(const float* __restrict__ x_rm, uint32_t d, uint32_t d4,
                                                         uint32_t k, const float* __restrict__ C,
                                                         const uint32_t* __restrict__ flagged,
                                                         const uint32_t* __restrict__ orig,
                                                         const TcIterDev* __restrict__ it, uint32_t* __restrict__ labels,
                                                         uint32_t* __restrict__ slabels, uint32_t* __restrict__ counts) {
    extern __shared__ float s_x[];  // [d][RECHECK_PTS]
    __shared__ float s_wv[8][RECHECK_PTS];
    __shared__ uint32_t s_wi[8][RECHECK_PTS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned int count = it->nflagged;
    const unsigned int groups = (count + RECHECK_PTS - 1) / RECHECK_PTS;
    for (unsigned int g = blockIdx.x; g < groups; g += gridDim.x) {
        const unsigned int q0 = g * RECHECK_PTS;
        const int np = (int)(count - q0 < (unsigned)RECHECK_PTS ? count - q0 : RECHECK_PTS);
        for (uint32_t e = threadIdx.x; e < d * RECHECK_PTS; e += blockDim.x) {
            const uint32_t f = e / RECHECK_PTS, i = e % RECHECK_PTS;
            s_x[e] = (int)i < np ? x_rm[(uint64_t)flagged[q0 + i] * d4 + f] : 0.0f;
        }
        __syncthreads();
        float bv[RECHECK_PTS];
        uint32_t bi[RECHECK_PTS];
#pragma unroll
        for (int i = 0; i < RECHECK_PTS; ++i) {
            bv[i] = FLT_MAX;
            bi[i] = NONE;
        }
        for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) {
            float acc[RECHECK_PTS];
#pragma unroll
            for (int i = 0; i < RECHECK_PTS; ++i) acc[i] = 0.0f;
            for (uint32_t f = 0; f < d; ++f) {
                const float cv = __ldg(C + (uint64_t)f * k + c);
                const float4* xf = reinterpret_cast<const float4*>(s_x + f * RECHECK_PTS);
#pragma unroll
                for (int i4 = 0; i4 < RECHECK_PTS / 4; ++i4) {
                    const float4 x = xf[i4];
                    float t = x.x - cv;
                    acc[4 * i4] = fmaf(t, t, acc[4 * i4]);
                    t = x.y - cv;
                    acc[4 * i4 + 1] = fmaf(t, t, acc[4 * i4 + 1]);
                    t = x.z - cv;
                    acc[4 * i4 + 2] = fmaf(t, t, acc[4 * i4 + 2]);
                    t = x.w - cv;
                    acc[4 * i4 + 3] = fmaf(t, t, acc[4 * i4 + 3]);
                }
            }
#pragma unroll
            for (int i = 0; i < RECHECK_PTS; ++i)
                if (acc[i] < bv[i]) {
                    bv[i] = acc[i];
                    bi[i] = c;
                }
        }
#pragma unroll
        for (int i = 0; i < RECHECK_PTS; ++i) {
            float v = bv[i];
            uint32_t x = bi[i];
            for (int o = 16; o > 0; o >>= 1) {
                const float ov = __shfl_xor_sync(0xffffffffu, v, o);
                const uint32_t oi = __shfl_xor_sync(0xffffffffu, x, o);
                if (ov < v || (ov == v && oi < x)) {
                    v = ov;
                    x = oi;
                }
            }
            if (lane == 0) {
                s_wv[warp][i] = v;
                s_wi[warp][i] = x;
            }
        }
        __syncthreads();
        if ((int)threadIdx.x < np) {
            const int i = threadIdx.x;
            float v = s_wv[0][i];
            uint32_t x = s_wi[0][i];
            for (int w = 1; w < 8; ++w)
                if (s_wv[w][i] < v || (s_wv[w][i] == v && s_wi[w][i] < x)) {
                    v = s_wv[w][i];
                    x = s_wi[w][i];
                }
            const uint32_t lab = x == NONE ? 0u : x;
            const uint32_t p = flagged[q0 + i];
            labels[orig[p]] = lab;
            slabels[p] = lab;
            count_label(counts, lab);
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// Centroid update: counting sort by label + segmented sums
// --------------------------------------------------------------------------

// From this call's counts (which share their array with the cursor):
// off[c] = first position of cluster c in label order (off[k] = n), the
// scatter cursor = off, and the counts added to the FP64 merge scratch's
// masses (which accumulate across calls in CKM_MODE_DEFER).  One CTA.
__global__ void __launch_bounds__(1024) tc_offsets_kernel(const uint32_t* counts, uint32_t k, uint32_t* __restrict__ off,
                                                          uint32_t* cursor, unsigned long long* __restrict__ msum) {
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0u;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < k; c0 += blockDim.x) {
        const uint32_t c = c0 + threadIdx.x;
        const uint32_t v = c < k ? counts[c] : 0u;
        uint32_t x = v;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t excl = s_carry + (warp > 0 ? s_warp[warp - 1] : 0u) + x - v;
        if (c < k) {
            off[c] = excl;
            cursor[c] = excl;  // same thread read counts[c] above
            if (v) msum[c] += v;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[k] = s_carry;
}

// perm[cursor[label]++] = p for a contiguous range of points per CTA: the
// CTA counts its labels in shared memory, reserves one range per label with a
// single global atomic, then places its points with shared-memory atomics.
// (Per-point global atomics on k counters serialise in L2: each counter
// receives n / k increments.)
__global__ void __launch_bounds__(1024) tc_scatter_local_kernel(const uint32_t* __restrict__ labels, uint64_t n,
                                                                uint32_t k, uint64_t per_cta,
                                                                uint32_t* __restrict__ cursor,
                                                                uint32_t* __restrict__ perm) {
    extern __shared__ uint32_t s_bin[];  // [k]
    const uint64_t p0 = (uint64_t)blockIdx.x * per_cta;
    const uint64_t p1 = p0 + per_cta < n ? p0 + per_cta : n;
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) s_bin[c] = 0u;
    __syncthreads();
    for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const uint32_t c = labels[p];
        if (c < k) atomicAdd(&s_bin[c], 1u);
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < k; c += blockDim.x)
        if (s_bin[c]) s_bin[c] = atomicAdd(&cursor[c], s_bin[c]);
    __syncthreads();
    for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const uint32_t c = labels[p];
        if (c >= k) continue;  // only after a failed labeling; never written out of bounds
        const uint32_t pos = atomicAdd(&s_bin[c], 1u);
        if (pos < n) perm[pos] = (uint32_t)p;
    }
}

// The same with per-point global atomics (lanes with equal labels share one),
// for k too large for a shared-memory histogram.
__global__ void __launch_bounds__(256) tc_scatter_kernel(const uint32_t* __restrict__ labels, uint64_t n, uint32_t k,
                                                         uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm) {
    const int lane = threadIdx.x & 31;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x; b < n; b += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = b + threadIdx.x;
        const bool in = p < n;
        const unsigned int active = __ballot_sync(0xffffffffu, in);
        if (!in) continue;
        const uint32_t c = labels[p];
        const unsigned int peers = __match_any_sync(active, c);
        if (c >= k) continue;  // only after a failed labeling; never written out of bounds
        const int leader = __ffs(peers) - 1;
        uint32_t pos = 0;
        if (lane == leader) pos = atomicAdd(&cursor[c], (uint32_t)__popc(peers));
        pos = __shfl_sync(peers, pos, leader) + __popc(peers & ((1u << lane) - 1u));
        if (pos < n) perm[pos] = (uint32_t)p;
    }
}

// hi + lo += v with an error-free transformation (Knuth's TwoSum).
__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float v) {
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// Per warp a slice of SEG positions of the label order: the rows of the
// points of one cluster are contiguous there, so each lane accumulates its
// features (float4 q = lane + 32 j of the row: features 4q..4q+3) as float
// pairs and merges them into the FP64 sums [d][k] only where the cluster
// changes.  ROWS rows are loaded before they are added, to keep loads in flight.
constexpr uint32_t SEG = 512;
constexpr int ROWS = 8;
template <int J>
__global__ void __launch_bounds__(256) tc_segment_sum_kernel(const float* __restrict__ x_rm, uint32_t d, uint32_t d4,
                                                             uint64_t n, uint32_t k, const uint32_t* __restrict__ perm,
                                                             const uint32_t* __restrict__ off,
                                                             double* __restrict__ sums) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t q4 = d4 / 4;  // float4 per row
    const uint64_t wid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    // positions past off[k] belong to no cluster (only after a failed labeling)
    const uint64_t total = __ldg(off + k) < n ? __ldg(off + k) : n;
    for (uint64_t s0 = wid * SEG; s0 < total; s0 += nw * SEG) {
        const uint64_t s1 = s0 + SEG < total ? s0 + SEG : total;
        uint32_t lo = 0, hi = k;  // cluster c with off[c] <= s0 < off[c + 1]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(off + mid) <= s0) lo = mid;
            else hi = mid;
        }
        uint32_t c = lo;
        uint64_t end = __ldg(off + c + 1);
        float ah[J][4], al[J][4];
#pragma unroll
        for (int j = 0; j < J; ++j)
#pragma unroll
            for (int t = 0; t < 4; ++t) ah[j][t] = al[j][t] = 0.0f;
        bool any = false;
        auto flush = [&]() {
            if (any) {
#pragma unroll
                for (int j = 0; j < J; ++j)
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const uint32_t f = 4u * (lane + 32u * j) + t;
                        if (f < d) atomicAdd(&sums[(uint64_t)f * k + c], (double)ah[j][t] + (double)al[j][t]);
                        ah[j][t] = al[j][t] = 0.0f;
                    }
            }
            any = false;
        };
        for (uint64_t b = s0; b < s1; b += 32) {
            const uint32_t cntq = (uint32_t)(s1 - b < 32 ? s1 - b : 32);
            const uint32_t myp = lane < cntq ? __ldg(perm + b + lane) : 0u;
            for (uint32_t i = 0; i < cntq; i += ROWS) {
                float4 v[ROWS][J];
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const uint32_t pr = __shfl_sync(0xffffffffu, myp, (i + r) & 31);
                    const bool ok = i + r < cntq && pr < n;
                    const float4* row = reinterpret_cast<const float4*>(x_rm + (uint64_t)(ok ? pr : 0u) * d4);
#pragma unroll
                    for (int j = 0; j < J; ++j) {
                        const uint32_t qq = lane + 32u * j;
                        v[r][j] = (ok && qq < q4) ? __ldg(row + qq) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    }
                }
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    if (i + r >= cntq) break;
                    const uint64_t qpos = b + i + r;
                    while (qpos >= end) {  // cluster boundary (empty clusters are skipped)
                        flush();
                        ++c;
                        end = __ldg(off + c + 1);
                    }
#pragma unroll
                    for (int j = 0; j < J; ++j) {
                        two_sum_add(ah[j][0], al[j][0], v[r][j].x);
                        two_sum_add(ah[j][1], al[j][1], v[r][j].y);
                        two_sum_add(ah[j][2], al[j][2], v[r][j].z);
                        two_sum_add(ah[j][3], al[j][3], v[r][j].w);
                    }
                    any = true;
                }
            }
        }
        flush();
    }
}

// Centroids from the FP64 sums (FINALIZE: sums / counts, 0/0 -> NaN for an
// empty cluster as in the reference; ACCUMULATE: centroids += sums), sums
// cleared for the next iteration.
__global__ void tc_finalize_sums_kernel(uint32_t d, uint32_t k, float* __restrict__ C, ScratchView sv, int mode) {
    const uint64_t kd = (uint64_t)k * d;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < kd; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(e % k);
        const double s = sv.sums[e];
        if (mode == CKM_MODE_FINALIZE) C[e] = (float)(s / (double)sv.masses[c]);
        else C[e] = C[e] + (float)s;
        sv.sums[e] = 0.0;
    }
}

__global__ void tc_finalize_masses_kernel(uint32_t k, uint32_t* __restrict__ masses, ScratchView sv, int mode) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < k; c += gridDim.x * blockDim.x) {
        const unsigned long long m = sv.masses[c];
        if (mode == CKM_MODE_FINALIZE) masses[c] = (uint32_t)m;
        else masses[c] = masses[c] + (uint32_t)m;
        sv.masses[c] = 0ull;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) sv.ctrl[0] = 0u;
}

// --------------------------------------------------------------------------
// Cluster-ordered point sets
// --------------------------------------------------------------------------

// dst row i = src row perm[i], with perm the label order of the last
// iteration (counting sort).  Points of one cluster then share 128-point
// tiles, so the lanes of a warp find their candidates in the same columns.
// The caller's indices move with the rows.  When that order does not cover
// all n points (a failed labeling) the rows are copied unchanged.
__global__ void __launch_bounds__(256) tc_sort_points_kernel(uint64_t n, uint32_t k, uint32_t d_pad, uint32_t d4,
                                                             const uint32_t* __restrict__ perm,
                                                             const uint32_t* __restrict__ off,
                                                             const uint4* __restrict__ sh, uint4* __restrict__ dh,
                                                             const float* __restrict__ sn, float* __restrict__ dn,
                                                             const float* __restrict__ se, float* __restrict__ de,
                                                             const float4* __restrict__ sr, float4* __restrict__ dr,
                                                             const uint32_t* __restrict__ so, uint32_t* __restrict__ dor) {
    const bool ordered = __ldg(off + k) == n;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t hrow = d_pad / 8, rrow = d4 / 4;  // 16-byte units per row
    for (uint64_t i = w0; i < n; i += nw) {
        uint64_t src = ordered ? __ldg(perm + i) : i;
        if (src >= n) src = i;
        for (uint32_t c = lane; c < hrow; c += 32) dh[i * hrow + c] = __ldg(sh + src * hrow + c);
        for (uint32_t c = lane; c < rrow; c += 32) dr[i * rrow + c] = __ldg(sr + src * rrow + c);
        if (lane == 0) {
            dn[i] = __ldg(sn + src);
            de[i] = __ldg(se + src);
            dor[i] = __ldg(so + src);
        }
    }
}

// --------------------------------------------------------------------------
// Host helpers
// --------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

// 2-D fp16 map over a K-major [rows][d_pad] matrix; box = 64 x box_rows with
// the 128-byte swizzle the MMA descriptors expect.
int make_map(CUtensorMap* m, const void* ptr, uint64_t rows, uint32_t d_pad, uint32_t box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return fail(CKM_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {d_pad, rows};
    cuuint64_t strides[1] = {(cuuint64_t)d_pad * 2};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? CKM_OK : fail(CKM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

int grid_for_n(uint64_t n, int block, int per_sm = 16) {
    uint64_t g = (n + block - 1) / block;
    const uint64_t cap = (uint64_t)device_info().sm_count * per_sm;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Shape of the label kernel: clusters per chunk and CTAs per SM.  One CTA
// per SM holds all 512 tensor-memory columns (two tiles x two buffers x 128
// clusters); with d_pad = 256 the chunks are 64 clusters to fit shared
// memory.  (Two CTAs per SM with 64-cluster chunks measured slower: one
// centroid stage each and twice the centroid traffic.)
uint32_t label_bn(uint32_t d_pad) { return d_pad <= 192 ? 128u : 64u; }
uint32_t label_ctas_per_sm(uint32_t) { return 1u; }

// Pipeline depth of the label kernel for a shape: two pair stages when they
// fit, then as many centroid stages as fit (at least one of each).
struct LabelCfg {
    uint32_t a_stages, b_stages, ctas_per_sm;
    size_t smem;
    bool ok;
};

template <int BN, bool CN_SMEM>
int label_static_smem(size_t* out) {
    static size_t cached[64] = {0};
    static bool have[64] = {false};
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 0 && dev < 64 && have[dev]) {
        *out = cached[dev];
        return CKM_OK;
    }
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, tc_label_kernel<BN, CN_SMEM>);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(tc_label)");
    e = cudaFuncSetAttribute(tc_label_kernel<BN, CN_SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(device_info().smem_optin - fa.sharedSizeBytes));
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(tc_label)");
    if (dev >= 0 && dev < 64) {
        cached[dev] = fa.sharedSizeBytes;
        have[dev] = true;
    }
    *out = fa.sharedSizeBytes;
    return CKM_OK;
}

LabelCfg label_cfg(uint32_t d_pad, uint32_t bn, uint32_t ctas, size_t static_smem, size_t extra = 0) {
    LabelCfg c{0, 0, ctas, 0, false};
    const DeviceInfo& di = device_info();
    const size_t per_cta = di.smem_per_sm / ctas;  // including the system's reservation
    const size_t limit = std::min(di.smem_optin, per_cta > di.smem_reserved ? per_cta - di.smem_reserved : 0);
    if (limit < static_smem + 1024) return c;
    const size_t budget = limit - static_smem - 1024;  // 1024: alignment of the swizzled tiles
    const size_t lists = (size_t)(CAP + 1) * EPI_THREADS * 8 + extra;
    const size_t a = (size_t)PAIR_M * d_pad * 2, b = (size_t)bn * d_pad * 2;
    uint32_t tries[8][2] = {{2, 4}, {2, 3}, {2, 2}, {1, 4}, {1, 3}, {1, 2}, {1, 1}, {1, 1}};
    // tuning: CKM_TC_STAGES="a,b" tries that depth first
    const char* env = std::getenv("CKM_TC_STAGES");
    unsigned ea = 0, eb = 0;
    if (env && std::sscanf(env, "%u,%u", &ea, &eb) == 2 && ea >= 1 && ea <= MAX_A_STAGES && eb >= 1 &&
        eb <= MAX_B_STAGES) {
        for (int i = 7; i > 0; --i) {
            tries[i][0] = tries[i - 1][0];
            tries[i][1] = tries[i - 1][1];
        }
        tries[0][0] = ea;
        tries[0][1] = eb;
    }
    for (const auto& t : tries) {
        const size_t need = t[0] * a + t[1] * b + lists;
        if (need <= budget) {
            c.a_stages = t[0];
            c.b_stages = t[1];
            c.smem = need + 1024;
            // no more than `ctas` CTAs per SM: together they own all the
            // tensor-memory columns
            const size_t floor_smem = di.smem_per_sm / (ctas + 1) + 1;
            if (c.smem + static_smem + di.smem_reserved < floor_smem)
                c.smem = floor_smem - static_smem - di.smem_reserved;
            c.ok = true;
            return c;
        }
    }
    return c;
}

}  // namespace

TcLayout tc_layout(uint64_t n, uint32_t d, uint32_t k) {
    TcLayout L;
    L.d_pad = (d + 63) / 64 * 64;
    L.d4 = (d + 3) / 4 * 4;
    L.bn = label_bn(L.d_pad);
    L.k_pad = (k + L.bn - 1) / L.bn * L.bn;
    L.n_pad = ((n > 0 ? n : 1) + PAIR_M - 1) / PAIR_M * PAIR_M;
    size_t off = 256;  // TcPointsHeader
    L.pts_half_off = off;
    off += align256((size_t)L.n_pad * L.d_pad * 2);
    L.pts_norm_off = off;
    off += align256((size_t)L.n_pad * 4);
    L.pts_err_off = off;
    off += align256((size_t)L.n_pad * 4);
    L.pts_rm_off = off;
    off += align256((size_t)n * L.d4 * 4);
    L.pts_orig_off = off;
    off += align256((size_t)n * 4);
    L.pts_total = off;
    off = 256;  // TcIterDev
    L.ws_cent_rm_off = off;
    off += align256((size_t)k * L.d4 * 4);
    L.ws_cent_half_off = off;
    off += align256((size_t)L.k_pad * L.d_pad * 2);
    L.ws_cn2_off = off;
    off += align256((size_t)L.k_pad * 4);
    L.ws_flagged_off = off;
    off += align256((size_t)n * 4);
    L.ws_off_off = off;
    off += align256(((size_t)k + 1) * 4);
    L.ws_cursor_off = off;
    off += align256((size_t)k * 4);
    L.ws_perm_off = off;
    off += align256((size_t)n * 4);
    L.ws_slabels_off = off;
    off += align256((size_t)n * 4);
    L.ws_res_pts_off = off;
    off += align256((size_t)n * 4);
    L.ws_res_cands_off = off;
    off += align256((size_t)n * CAP * 4);
    L.ws_total = off;
    return L;
}

bool tc_supported(uint32_t d, uint32_t k) {
    const DeviceInfo& di = device_info();
    if (di.cc_major != 10 || d == 0 || k == 0) return false;
    const uint32_t d_pad = (d + 63) / 64 * 64;
    if (d_pad > 256) return false;
    // the label kernel's static shared memory is under 1 KB
    return label_cfg(d_pad, label_bn(d_pad), label_ctas_per_sm(d_pad), 1024, CN_SMEM_MAX * sizeof(float)).ok;
}

int tc_prepare_points(const float* P, uint64_t n, uint32_t d, void* tc_points, int precision, cudaStream_t s) {
    const TcLayout L = tc_layout(n, d, 1);
    char* b = static_cast<char*>(tc_points);
    TcPointsHeader* hdr = reinterpret_cast<TcPointsHeader*>(b);
    // header, 2-byte operand rows and norms start zeroed: padding rows stay zero
    cudaError_t e = cudaMemsetAsync(b, 0, L.pts_rm_off, s);
    // the operand type (0 or 1) in the header's low byte of `precision`
    if (e == cudaSuccess && precision)
        e = cudaMemsetAsync(reinterpret_cast<char*>(&hdr->precision), precision, 1, s);
    if (e != cudaSuccess) return cuda_fail(e, "tc_prepare_points memset");
    if (n == 0) return CKM_OK;
    tc_points_maxabs_kernel<<<grid_for_n(n * d, 256, 8), 256, 0, s>>>(P, n * d, hdr);
    count_launch();
    tc_points_convert_kernel<<<grid_for_n(n, 32, 16), 256, (size_t)d * 33 * sizeof(float), s>>>(
        P, n, d, L.d_pad, L.d4, hdr, reinterpret_cast<uint16_t*>(b + L.pts_half_off),
        reinterpret_cast<float*>(b + L.pts_norm_off), reinterpret_cast<float*>(b + L.pts_err_off),
        reinterpret_cast<float*>(b + L.pts_rm_off), reinterpret_cast<uint32_t*>(b + L.pts_orig_off));
    count_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "tc_prepare_points launch");
}

int tc_sort_points(uint64_t n, uint32_t d, uint32_t k, const void* src, void* dst, const void* workspace,
                   cudaStream_t s) {
    const TcLayout L = tc_layout(n, d, k);
    const char* sb = static_cast<const char*>(src);
    char* db = static_cast<char*>(dst);
    const char* ws = static_cast<const char*>(workspace);
    // header as is; tile padding rows and their norms zero
    cudaError_t e = cudaMemcpyAsync(db, sb, 256, cudaMemcpyDeviceToDevice, s);
    const size_t hrow = (size_t)L.d_pad * 2;
    if (e == cudaSuccess && L.n_pad > n)
        e = cudaMemsetAsync(db + L.pts_half_off + n * hrow, 0, (L.n_pad - n) * hrow, s);
    if (e == cudaSuccess && L.n_pad > n) e = cudaMemsetAsync(db + L.pts_norm_off + n * 4, 0, (L.n_pad - n) * 4, s);
    if (e == cudaSuccess && L.n_pad > n) e = cudaMemsetAsync(db + L.pts_err_off + n * 4, 0, (L.n_pad - n) * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "tc_sort_points copy");
    if (n == 0) return CKM_OK;
    tc_sort_points_kernel<<<grid_for_n(n * 32, 256), 256, 0, s>>>(
        n, k, L.d_pad, L.d4, reinterpret_cast<const uint32_t*>(ws + L.ws_perm_off),
        reinterpret_cast<const uint32_t*>(ws + L.ws_off_off), reinterpret_cast<const uint4*>(sb + L.pts_half_off),
        reinterpret_cast<uint4*>(db + L.pts_half_off), reinterpret_cast<const float*>(sb + L.pts_norm_off),
        reinterpret_cast<float*>(db + L.pts_norm_off), reinterpret_cast<const float*>(sb + L.pts_err_off),
        reinterpret_cast<float*>(db + L.pts_err_off), reinterpret_cast<const float4*>(sb + L.pts_rm_off),
        reinterpret_cast<float4*>(db + L.pts_rm_off), reinterpret_cast<const uint32_t*>(sb + L.pts_orig_off),
        reinterpret_cast<uint32_t*>(db + L.pts_orig_off));
    count_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "tc_sort_points launch");
}

template <int BN, bool CN_SMEM>
static int launch_label(const TcLayout& L, const LabelParams& prm, const void* pts_half, const void* cent_half,
                        cudaStream_t s) {
    size_t st = 0;
    int rc = label_static_smem<BN, CN_SMEM>(&st);
    if (rc) return rc;
    const LabelCfg cfg =
        label_cfg(L.d_pad, BN, label_ctas_per_sm(L.d_pad), st, CN_SMEM ? (size_t)L.k_pad * sizeof(float) : 0);
    if (!cfg.ok) return fail(CKM_ERR_UNSUPPORTED, "tensor-core label kernel: shared memory too small");
    CUtensorMap tm_a, tm_b;
    if ((rc = make_map(&tm_a, pts_half, L.n_pad, L.d_pad, PAIR_M))) return rc;
    if ((rc = make_map(&tm_b, cent_half, L.k_pad, L.d_pad, BN))) return rc;
    LabelParams p = prm;
    p.a_stages = cfg.a_stages;
    p.b_stages = cfg.b_stages;
    const uint32_t slots = (uint32_t)device_info().sm_count * cfg.ctas_per_sm;
    const uint32_t grid = p.num_pairs < slots ? p.num_pairs : slots;
    tc_label_kernel<BN, CN_SMEM><<<grid, LABEL_THREADS, cfg.smem, s>>>(tm_a, tm_b, p);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "tc_label launch");
}

static int launch_label_for(const TcLayout& L, const LabelParams& prm, const void* pts_half, const void* cent_half,
                            cudaStream_t s) {
    const bool cn_smem = L.k_pad <= CN_SMEM_MAX;
    if (L.bn == 128)
        return cn_smem ? launch_label<128, true>(L, prm, pts_half, cent_half, s)
                       : launch_label<128, false>(L, prm, pts_half, cent_half, s);
    return cn_smem ? launch_label<64, true>(L, prm, pts_half, cent_half, s)
                   : launch_label<64, false>(L, prm, pts_half, cent_half, s);
}

int tc_iteration(const TcArgs& a, cudaStream_t s) {
    if (!tc_supported(a.d, a.k)) return fail(CKM_ERR_UNSUPPORTED, "tensor-core path: unsupported shape or device");
    if (a.n >= 0xffffffffull) return fail(CKM_ERR_UNSUPPORTED, "tensor-core path: at most 2^32 - 2 points per call");
    const TcLayout L = tc_layout(a.n, a.d, a.k);
    const char* pb = static_cast<const char*>(a.tc_points);
    char* ws = static_cast<char*>(a.workspace);
    TcIterDev* it = reinterpret_cast<TcIterDev*>(ws);
    float* cent_rm = reinterpret_cast<float*>(ws + L.ws_cent_rm_off);
    uint16_t* cent_half = reinterpret_cast<uint16_t*>(ws + L.ws_cent_half_off);
    float* cn2 = reinterpret_cast<float*>(ws + L.ws_cn2_off);
    uint32_t* flagged = reinterpret_cast<uint32_t*>(ws + L.ws_flagged_off);
    uint32_t* off = reinterpret_cast<uint32_t*>(ws + L.ws_off_off);
    uint32_t* cursor = reinterpret_cast<uint32_t*>(ws + L.ws_cursor_off);  // counts, then scatter cursor
    uint32_t* perm = reinterpret_cast<uint32_t*>(ws + L.ws_perm_off);
    uint32_t* slabels = reinterpret_cast<uint32_t*>(ws + L.ws_slabels_off);  // labels in the set's order

    cudaError_t e = cudaMemsetAsync(it, 0, 256, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, (size_t)a.k * 4, s);
    if (e != cudaSuccess) return cuda_fail(e, "tc memset");
    const int cgrid = (int)((L.k_pad + 255) / 256);
    tc_centroid_stats_kernel<<<cgrid, 256, 0, s>>>(a.centroids, a.k, a.d, L.k_pad, L.d4, cent_rm, cn2, it);
    count_launch();
    tc_centroid_pack_kernel<<<cgrid, 256, 0, s>>>(a.centroids, a.k, a.d, L.k_pad, L.d_pad, cn2, cent_half,
                                                  reinterpret_cast<const TcPointsHeader*>(pb), it);
    count_launch();
    tc_params_kernel<<<1, 1, 0, s>>>(a.d, L.d_pad, reinterpret_cast<const TcPointsHeader*>(pb), it);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "tc centroid launch");

    if (a.n > 0) {
        LabelParams prm;
        prm.norms = reinterpret_cast<const float*>(pb + L.pts_norm_off);
        prm.errn = reinterpret_cast<const float*>(pb + L.pts_err_off);
        prm.x_rm = reinterpret_cast<const float*>(pb + L.pts_rm_off);
        prm.orig = reinterpret_cast<const uint32_t*>(pb + L.pts_orig_off);
        prm.precision = &reinterpret_cast<const TcPointsHeader*>(pb)->precision;
        prm.slabels = slabels;
        prm.res_pts = reinterpret_cast<uint32_t*>(ws + L.ws_res_pts_off);
        prm.res_cands = reinterpret_cast<uint32_t*>(ws + L.ws_res_cands_off);
        prm.c_rm = cent_rm;
        prm.cn2 = cn2;
        prm.it = it;
        prm.labels = a.labels;
        prm.counts = cursor;
        prm.flagged = flagged;
        prm.n = a.n;
        prm.d = a.d;
        prm.d4 = L.d4;
        prm.d_pad = L.d_pad;
        prm.k = a.k;
        prm.chunks = L.k_pad / L.bn;
        prm.num_pairs = (uint32_t)(L.n_pad / PAIR_M);
        prm.a_stages = prm.b_stages = 1;
        const int rc = launch_label_for(L, prm, pb + L.pts_half_off, cent_half, s);
        if (rc) return rc;
        tc_resolve_kernel<<<device_info().sm_count * 8, 256, 0, s>>>(prm.x_rm, cent_rm, a.d, L.d4, prm.res_pts,
                                                                     prm.res_cands, prm.orig, it, flagged, a.labels,
                                                                     slabels, cursor);
        count_launch();
        tc_recheck_kernel<<<device_info().sm_count * 4, 256, (size_t)a.d * RECHECK_PTS * sizeof(float), s>>>(
            prm.x_rm, a.d, L.d4, a.k, a.centroids, flagged, prm.orig, it, a.labels, slabels, cursor);
        count_launch();
    }
    tc_offsets_kernel<<<1, 1024, 0, s>>>(cursor, a.k, off, cursor, a.scratch.masses);
    count_launch();
    if (a.n > 0) {
        const size_t bins = (size_t)a.k * sizeof(uint32_t);
        if (bins <= 48 * 1024) {
            const uint64_t ctas = (uint64_t)device_info().sm_count * 2;
            const uint64_t per = (a.n + ctas - 1) / ctas;
            tc_scatter_local_kernel<<<(unsigned)((a.n + per - 1) / per), 1024, bins, s>>>(slabels, a.n, a.k, per,
                                                                                         cursor, perm);
        } else {
            tc_scatter_kernel<<<grid_for_n(a.n, 256), 256, 0, s>>>(slabels, a.n, a.k, cursor, perm);
        }
        count_launch();
        const uint64_t warps = (a.n + SEG - 1) / SEG;
        const int sgrid = grid_for_n(warps * 32, 256);
        const float* x_rm = reinterpret_cast<const float*>(pb + L.pts_rm_off);
        if (L.d4 <= 128)
            tc_segment_sum_kernel<1><<<sgrid, 256, 0, s>>>(x_rm, a.d, L.d4, a.n, a.k, perm, off, a.scratch.sums);
        else
            tc_segment_sum_kernel<2><<<sgrid, 256, 0, s>>>(x_rm, a.d, L.d4, a.n, a.k, perm, off, a.scratch.sums);
        count_launch();
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "tc update launch");
    if (a.mode != CKM_MODE_DEFER) {
        tc_finalize_sums_kernel<<<grid_for_n((uint64_t)a.k * a.d, 256), 256, 0, s>>>(a.d, a.k, a.new_centroids,
                                                                                    a.scratch, a.mode);
        count_launch();
        tc_finalize_masses_kernel<<<(a.k + 255) / 256, 256, 0, s>>>(a.k, a.masses, a.scratch, a.mode);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "tc finalize launch");
    }
    if (a.stats) {
        e = cudaMemcpyAsync(a.stats, it, 2 * sizeof(unsigned int), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "tc stats copy");
    }
    return CKM_OK;
}

}  // namespace ckm
