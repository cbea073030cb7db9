// Tensor-core Lloyd iteration for large k*d (tcgen05, sm_100 family).
//
// Distances as a GEMM: score(x, c) = |c|^2 - 2 x.c; argmin over c of the
// score is the argmin of |x - c|^2.  Per 128-point tile (one CTA):
//   - the points' bf16 copy (K-major [n][d_pad], made once per run by
//     tc_prepare_points) arrives by TMA in the 128-byte swizzled layout;
//   - clusters go in chunks of 256: TMA loads the bf16 centroid chunk, one
//     elected thread issues d_pad/16 tcgen05.mma (M=128, N=256, K=16, f32
//     accumulation in tensor memory), commit -> mbarrier;
//   - each thread owns one point (= one TMEM lane), reads its 256 scores with
//     tcgen05.ld and keeps its TOPK + 1 smallest scores (TOPK clusters);
//   - a rigorous per-point error bound covers the bf16 rounding of both
//     operands (2^-9 relative each), the f32 accumulation and the FP32
//     rounding of the reference distance itself.  A cluster whose score is
//     more than twice the bound above the best score cannot win the exact
//     FP32 comparison of kmeans_naive.cpp:48-63.  So: one cluster within the
//     bound -> that is the reference's label; 2..TOPK clusters within it ->
//     the thread computes exactly those distances with the reference
//     arithmetic (ascending cluster order, strict '<'); more -> the point
//     goes on a list for tc_recheck_kernel (all clusters, exact);
//   - resolved points add their FP32 coordinates into the FP64 scratch.
// Empty (NaN) and padding clusters get zero rows and |c|^2 = +inf, so they
// never win, as NaN never wins in the reference.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "ckm_device.cuh"
#include "ckm_internal.h"
#include "ckm_tc.h"
#include "ckm_umma.cuh"

namespace ckm {
namespace {

constexpr int TC_M = 128;        // points per CTA (TMEM lanes)
constexpr int TC_N = 256;        // clusters per chunk (TMEM columns)
constexpr int TC_THREADS = 128;  // one thread per point
constexpr int TOPK = 8;          // candidates resolved in the kernel by exact arithmetic

// --------------------------------------------------------------------------
// Preparation kernels
// --------------------------------------------------------------------------

// bf16 copy of the points, K-major [n][d_pad] (zero padded), and per point
// the norm of the bf16 vector.
__global__ void tc_prepare_points_kernel(const float* __restrict__ P, uint64_t n, uint32_t d, uint32_t d_pad,
                                         __nv_bfloat16* __restrict__ out, float* __restrict__ norms) {
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        __nv_bfloat16* row = out + p * d_pad;
        for (uint32_t f = 0; f < d_pad; ++f) {
            const float v = f < d ? P[(uint64_t)f * n + p] : 0.0f;
            const __nv_bfloat16 b = __float2bfloat16_rn(v);
            row[f] = b;
            const double bv = (double)__bfloat162float(b);
            s += bv * bv;
        }
        norms[p] = (float)sqrt(s);
    }
}

// Per iteration: bf16 centroids K-major [k_pad][d_pad] (NaN and padding
// rows zeroed), |c|^2 (+inf for those rows), and max |c| over valid rows.
__global__ void tc_prepare_centroids_kernel(const float* __restrict__ C, uint32_t k, uint32_t d, uint32_t k_pad,
                                            uint32_t d_pad, __nv_bfloat16* __restrict__ out,
                                            float* __restrict__ cnorm2, unsigned int* __restrict__ cmax_bits,
                                            float* __restrict__ rowmajor) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < k_pad; c += gridDim.x * blockDim.x) {
        bool valid = c < k;
        double s = 0.0;
        if (valid) {
            for (uint32_t f = 0; f < d; ++f) {
                const float v = C[(uint64_t)f * k + c];
                if (!(v == v) || isinf(v)) valid = false;
                s += (double)v * (double)v;
            }
        }
        __nv_bfloat16* row = out + (uint64_t)c * d_pad;
        for (uint32_t f = 0; f < d_pad; ++f)
            row[f] = __float2bfloat16_rn((valid && f < d) ? C[(uint64_t)f * k + c] : 0.0f);
        cnorm2[c] = valid ? (float)s : __int_as_float(0x7f800000);
        if (c < k)  // FP32 row-major copy: one candidate's features are contiguous
            for (uint32_t f = 0; f < d; ++f) rowmajor[(uint64_t)c * d + f] = C[(uint64_t)f * k + c];
        if (valid) atomicMax(cmax_bits, __float_as_uint((float)sqrt(s)));  // non-negative floats order as uints
    }
}

// --------------------------------------------------------------------------
// Labeling kernel
// --------------------------------------------------------------------------
struct TcParams {
    const float* points;      // FP32 column-major [d][n] (sums, exact candidate distances)
    const float* centroids;   // FP32 row-major [k][d] copy (exact candidate distances)
    const float* norms;       // |x~| per point
    const float* cnorm2;      // [k_pad]
    const unsigned int* cmax_bits;
    uint32_t* labels;
    uint32_t* flagged;        // indices of points for the exact recheck
    unsigned int* nflagged;
    unsigned int* error;      // nonzero: a bounded wait ran out
    double* sums;
    unsigned long long* msum;
    uint64_t n;
    uint32_t d, k, d_pad, k_pad;
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_label_kernel(const __grid_constant__ CUtensorMap tm_points, const __grid_constant__ CUtensorMap tm_cent,
                    const TcParams prm) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar_a, bar_b, bar_mma;
    __shared__ uint32_t tmem_base;
    __shared__ float s_cn[TC_N];
    __shared__ unsigned int s_fail;

    const uint32_t raw = umma::smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* sA = smem_raw + (base - raw);              // TC_M x d_pad bf16
    unsigned char* sB = sA + (size_t)TC_M * prm.d_pad * 2;    // TC_N x d_pad bf16
    const uint32_t kblocks = prm.d_pad / 64;
    const uint32_t a_bytes = TC_M * prm.d_pad * 2, b_bytes = TC_N * prm.d_pad * 2;
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint64_t p0 = (uint64_t)blockIdx.x * TC_M;

    if (warp == 0) umma::tmem_alloc(umma::smem_u32(&tmem_base), TC_N);
    if (tid == 0) {
        umma::mbar_init(umma::smem_u32(&bar_a), 1);
        umma::mbar_init(umma::smem_u32(&bar_b), 1);
        umma::mbar_init(umma::smem_u32(&bar_mma), 1);
        umma::mbar_fence_init();
        s_fail = 0u;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = umma::idesc_bf16_f32(TC_M, TC_N);

    if (tid == 0) {
        umma::mbar_arrive_expect_tx(umma::smem_u32(&bar_a), a_bytes);
        for (uint32_t kb = 0; kb < kblocks; ++kb)
            umma::tma_load_2d(umma::smem_u32(sA) + kb * TC_M * 128, &tm_points, (int)(kb * 64), (int)p0,
                              umma::smem_u32(&bar_a));
        umma::mbar_arrive_expect_tx(umma::smem_u32(&bar_b), b_bytes);
        for (uint32_t kb = 0; kb < kblocks; ++kb)
            umma::tma_load_2d(umma::smem_u32(sB) + kb * TC_N * 128, &tm_cent, (int)(kb * 64), 0,
                              umma::smem_u32(&bar_b));
    }

    // the TOPK + 1 smallest scores (ascending) and the clusters of the first TOPK
    float top[TOPK + 1];
    uint32_t top_i[TOPK];
#pragma unroll
    for (int t = 0; t <= TOPK; ++t) top[t] = __int_as_float(0x7f800000);
#pragma unroll
    for (int t = 0; t < TOPK; ++t) top_i[t] = 0xffffffffu;
    const uint32_t nchunks = prm.k_pad / TC_N;
    bool ok = true;
    for (uint32_t j = 0; j < nchunks; ++j) {
        for (uint32_t i = tid; i < TC_N; i += TC_THREADS) s_cn[i] = prm.cnorm2[j * TC_N + i];
        if (tid == 0) {
            bool loaded = (j > 0 || umma::mbar_wait(umma::smem_u32(&bar_a), 0)) &&
                          umma::mbar_wait(umma::smem_u32(&bar_b), j & 1u);
            if (loaded) {
                for (uint32_t ks = 0; ks < prm.d_pad / 16; ++ks) {
                    const uint32_t kb = ks / 4, sub = ks % 4;
                    const uint64_t ad = umma::sw128_desc(umma::smem_u32(sA) + kb * TC_M * 128 + sub * 32);
                    const uint64_t bd = umma::sw128_desc(umma::smem_u32(sB) + kb * TC_N * 128 + sub * 32);
                    umma::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
                }
                umma::mma_commit(umma::smem_u32(&bar_mma));
            } else {
                s_fail = 1u;
            }
        }
        __syncthreads();
        if (s_fail) {
            ok = false;
            break;
        }
        if (!umma::mbar_wait(umma::smem_u32(&bar_mma), j & 1u)) {
            s_fail = 1u;  // benign race: every writer stores 1
        }
        __syncthreads();
        if (s_fail) {
            ok = false;
            break;
        }
        umma::fence_after_sync();
        // the MMA has consumed the centroid chunk: prefetch the next one while scoring
        if (tid == 0 && j + 1 < nchunks) {
            umma::mbar_arrive_expect_tx(umma::smem_u32(&bar_b), b_bytes);
            for (uint32_t kb = 0; kb < kblocks; ++kb)
                umma::tma_load_2d(umma::smem_u32(sB) + kb * TC_N * 128, &tm_cent, (int)(kb * 64),
                                  (int)((j + 1) * TC_N), umma::smem_u32(&bar_b));
        }
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < TC_N; c0 += 16) {
            float v[16];
            umma::tmem_ld16(tmem + lane_base + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                float s = fmaf(-2.0f, v[i], s_cn[c0 + i]);
                if (s < top[TOPK]) {  // rare after the first clusters: one compare per score
                    uint32_t c = j * TC_N + c0 + i;
#pragma unroll
                    for (int t = 0; t < TOPK; ++t) {
                        if (s < top[t]) {
                            const float tv = top[t];
                            const uint32_t ti = top_i[t];
                            top[t] = s;
                            top_i[t] = c;
                            s = tv;
                            c = ti;
                        }
                    }
                    top[TOPK] = fminf(top[TOPK], s);
                }
            }
        }
        umma::fence_before_sync();
        __syncthreads();  // TMEM and s_cn are reused by the next chunk
    }

    if (ok) {
        const uint64_t p = p0 + tid;
        if (p < prm.n) {
            // certificate (see the file comment for the derivation)
            const float xn = prm.norms[p] * 1.004f;
            const float cm = __uint_as_float(*prm.cmax_bits) * 1.0001f;
            const float mag = fmaxf(fabsf(top[0]), fabsf(top[TOPK]));
            const float bound = 0.0081f * xn * cm + 1.6e-5f * (xn + cm) * (xn + cm) + 1.2e-7f * (cm * cm + mag);
            // candidates: clusters whose score is within twice the bound of the
            // best; every other cluster is certified to lose the exact FP32
            // comparison against the best candidate
            const float thr = top[0] + 2.0f * bound;
            uint32_t label = 0xffffffffu;
            if (top[0] < __int_as_float(0x7f800000) && top[TOPK] > thr && top_i[0] < prm.k) {
                if (!(top[1] <= thr)) {
                    label = top_i[0];  // a single candidate
                } else {
                    // 2..TOPK candidates: the reference arithmetic on just those,
                    // visited in ascending cluster order (strict '<' keeps the
                    // lowest index among equal distances)
                    uint32_t cand[TOPK];
                    int nc = 0;
#pragma unroll
                    for (int t = 0; t < TOPK; ++t)
                        if (top[t] <= thr && top_i[t] < prm.k) cand[nc++] = top_i[t];
                    for (int a = 1; a < nc; ++a)
                        for (int b = a; b > 0 && cand[b - 1] > cand[b]; --b) {
                            const uint32_t tmp = cand[b];
                            cand[b] = cand[b - 1];
                            cand[b - 1] = tmp;
                        }
                    float bv = FLT_MAX;
                    uint32_t bi = 0xffffffffu;
                    for (int a = 0; a < nc; ++a) {
                        const uint32_t c = cand[a];
                        float acc = 0.0f;
                        const float* crow = prm.centroids + (uint64_t)c * prm.d;
                        for (uint32_t f = 0; f < prm.d; ++f) {
                            const float t = __ldg(prm.points + (uint64_t)f * prm.n + p) - __ldg(crow + f);
                            acc = fmaf(t, t, acc);
                        }
                        if (acc < bv) {
                            bv = acc;
                            bi = c;
                        }
                    }
                    label = bi;  // 0xffffffff (nothing below FLT_MAX) -> full recheck
                }
            }
            if (label != 0xffffffffu) {
                prm.labels[p] = label;
                for (uint32_t f = 0; f < prm.d; ++f)
                    atomicAdd(&prm.sums[(uint64_t)f * prm.k + label], (double)__ldg(prm.points + (uint64_t)f * prm.n + p));
                atomicAdd(&prm.msum[label], 1ull);
            } else {
                const unsigned int slot = atomicAdd(prm.nflagged, 1u);
                prm.flagged[slot] = (uint32_t)p;
            }
        }
    } else if (tid == 0) {
        atomicExch(prm.error, 1u);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, TC_N);
}

// --------------------------------------------------------------------------
// Exact recheck of flagged points: the reference arithmetic over all
// clusters (t = x_f - c_f, acc = fma(t, t, acc) for f ascending; strict '<';
// lowest index among equal minima; NaN never wins; label 0 when nothing is
// below FLT_MAX), one CTA per point.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) tc_recheck_kernel(const float* __restrict__ P, uint64_t n, uint32_t d,
                                                         uint32_t k, const float* __restrict__ C,
                                                         const uint32_t* __restrict__ flagged,
                                                         const unsigned int* __restrict__ nflagged,
                                                         uint32_t* __restrict__ labels, double* __restrict__ sums,
                                                         unsigned long long* __restrict__ msum) {
    extern __shared__ float s_x[];
    __shared__ float s_bv[256];
    __shared__ uint32_t s_bi[256];
    const unsigned int count = *nflagged;
    for (unsigned int q = blockIdx.x; q < count; q += gridDim.x) {
        const uint64_t p = flagged[q];
        for (uint32_t f = threadIdx.x; f < d; f += blockDim.x) s_x[f] = P[(uint64_t)f * n + p];
        __syncthreads();
        float bv = FLT_MAX;
        uint32_t bi = 0xffffffffu;
        for (uint32_t c = threadIdx.x; c < k; c += blockDim.x) {
            float acc = 0.0f;
            for (uint32_t f = 0; f < d; ++f) {
                const float t = s_x[f] - C[(uint64_t)f * k + c];
                acc = fmaf(t, t, acc);
            }
            if (acc < bv) {
                bv = acc;
                bi = c;
            }
        }
        s_bv[threadIdx.x] = bv;
        s_bi[threadIdx.x] = bi;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int)threadIdx.x < o) {
                const float ov = s_bv[threadIdx.x + o];
                const uint32_t oi = s_bi[threadIdx.x + o];
                if (ov < s_bv[threadIdx.x] || (ov == s_bv[threadIdx.x] && oi < s_bi[threadIdx.x])) {
                    s_bv[threadIdx.x] = ov;
                    s_bi[threadIdx.x] = oi;
                }
            }
            __syncthreads();
        }
        const uint32_t lab = s_bi[0] == 0xffffffffu ? 0u : s_bi[0];
        if (threadIdx.x == 0) {
            labels[p] = lab;
            atomicAdd(&msum[lab], 1ull);
        }
        for (uint32_t f = threadIdx.x; f < d; f += blockDim.x) atomicAdd(&sums[(uint64_t)f * k + lab], (double)s_x[f]);
        __syncthreads();
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

// 2-D bf16 map over a K-major [rows][d_pad] matrix; box = 64 x box_rows with
// 128-byte swizzle.
int make_map(CUtensorMap* m, const void* ptr, uint64_t rows, uint32_t d_pad, uint32_t box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return fail(CKM_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {d_pad, rows};
    cuuint64_t strides[1] = {(cuuint64_t)d_pad * 2};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? CKM_OK : fail(CKM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

int grid_for_n(uint64_t n, int block) {
    uint64_t g = (n + block - 1) / block;
    const uint64_t cap = (uint64_t)device_info().sm_count * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

TcLayout tc_layout(uint64_t n, uint32_t d, uint32_t k) {
    TcLayout L;
    L.d_pad = (d + 63) / 64 * 64;
    L.k_pad = (k + TC_N - 1) / TC_N * TC_N;
    L.n_pad = (n + TC_M - 1) / TC_M * TC_M;
    auto a = [](size_t v) { return (v + 255) & ~size_t(255); };
    size_t off = 0;
    L.cent_rm_off = off;
    off += a((size_t)k * d * 4);
    L.cent_bf16_off = off;
    off += a((size_t)L.k_pad * L.d_pad * 2);
    L.cnorm2_off = off;
    off += a((size_t)L.k_pad * 4);
    L.cmax_off = off;
    off += 256;
    L.flagged_off = off;
    off += a((size_t)n * 4);
    L.counters_off = off;
    off += 256;
    L.total = off;
    L.points_bf16_bytes = (size_t)L.n_pad * L.d_pad * 2;
    L.norms_bytes = (size_t)L.n_pad * 4;
    return L;
}

bool tc_supported(uint32_t d, uint32_t k) {
    const DeviceInfo& di = device_info();
    if (di.cc_major != 10) return false;
    const uint32_t d_pad = (d + 63) / 64 * 64;
    if (d_pad == 0 || d_pad > 256) return false;
    const size_t smem = (size_t)(TC_M + TC_N) * d_pad * 2 + 1024;
    return smem <= di.smem_optin - 4096 && k >= 1;
}

int tc_prepare_points(const float* P, uint64_t n, uint32_t d, void* points_bf16, float* norms, cudaStream_t s) {
    const TcLayout L = tc_layout(n, d, 1);
    // rows past n (tile padding) are zeroed once
    cudaError_t e = cudaMemsetAsync(points_bf16, 0, L.points_bf16_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(norms, 0, L.norms_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "tc_prepare_points memset");
    tc_prepare_points_kernel<<<grid_for_n(n, 256), 256, 0, s>>>(P, n, d, L.d_pad,
                                                                reinterpret_cast<__nv_bfloat16*>(points_bf16), norms);
    count_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "tc_prepare_points launch");
}

int tc_iteration(const TcArgs& a, cudaStream_t s) {
    const TcLayout L = tc_layout(a.n, a.d, a.k);
    if (!tc_supported(a.d, a.k)) return fail(CKM_ERR_UNSUPPORTED, "tensor-core path: unsupported shape or device");
    char* ws = static_cast<char*>(a.workspace);
    __nv_bfloat16* cent_bf16 = reinterpret_cast<__nv_bfloat16*>(ws + L.cent_bf16_off);
    float* cent_rm = reinterpret_cast<float*>(ws + L.cent_rm_off);
    float* cnorm2 = reinterpret_cast<float*>(ws + L.cnorm2_off);
    unsigned int* cmax_bits = reinterpret_cast<unsigned int*>(ws + L.cmax_off);
    uint32_t* flagged = reinterpret_cast<uint32_t*>(ws + L.flagged_off);
    unsigned int* counters = reinterpret_cast<unsigned int*>(ws + L.counters_off);  // [0] nflagged, [1] error

    cudaError_t e = cudaMemsetAsync(cmax_bits, 0, 256, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 256, s);
    if (e != cudaSuccess) return cuda_fail(e, "tc memset");
    tc_prepare_centroids_kernel<<<(L.k_pad + 255) / 256, 256, 0, s>>>(a.centroids, a.k, a.d, L.k_pad, L.d_pad,
                                                                      cent_bf16, cnorm2, cmax_bits, cent_rm);
    count_launch();

    CUtensorMap tm_p, tm_c;
    int st = make_map(&tm_p, a.points_bf16, L.n_pad, L.d_pad, TC_M);
    if (st) return st;
    if ((st = make_map(&tm_c, cent_bf16, L.k_pad, L.d_pad, TC_N))) return st;

    TcParams prm;
    prm.points = a.points;
    prm.centroids = cent_rm;
    prm.norms = a.norms;
    prm.cnorm2 = cnorm2;
    prm.cmax_bits = cmax_bits;
    prm.labels = a.labels;
    prm.flagged = flagged;
    prm.nflagged = counters;
    prm.error = counters + 1;
    prm.sums = a.scratch.sums;
    prm.msum = a.scratch.masses;
    prm.n = a.n;
    prm.d = a.d;
    prm.k = a.k;
    prm.d_pad = L.d_pad;
    prm.k_pad = L.k_pad;
    // at least 100 KB so no more than two CTAs share an SM: each holds 256 of
    // the SM's 512 tensor-memory columns
    size_t smem = (size_t)(TC_M + TC_N) * L.d_pad * 2 + 1024;
    if (smem < 100 * 1024) smem = 100 * 1024;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> g(mu);
        static bool done[64] = {false};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev >= 0 && dev < 64 && !done[dev]) {
            cudaFuncAttributes fa;
            e = cudaFuncGetAttributes(&fa, tc_label_kernel);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(tc_label_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(device_info().smem_optin - fa.sharedSizeBytes));
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(tc_label)");
            done[dev] = true;
        }
    }
    const uint32_t tiles = (uint32_t)(L.n_pad / TC_M);
    if (tiles > 0) {
        tc_label_kernel<<<tiles, TC_THREADS, smem, s>>>(tm_p, tm_c, prm);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "tc_label launch");
    }
    const uint32_t rgrid = (uint32_t)device_info().sm_count * 8;
    tc_recheck_kernel<<<rgrid, 256, a.d * sizeof(float), s>>>(a.points, a.n, a.d, a.k, a.centroids, flagged, counters,
                                                             a.labels, a.scratch.sums, a.scratch.masses);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "tc_recheck launch");
    if (a.mode != CKM_MODE_DEFER) {
        st = launch_finalize_f32(a.d, a.k, a.new_centroids, a.masses, a.scratch, a.mode, s);
        if (st) return st;
    }
    if (a.stats) {
        e = cudaMemcpyAsync(a.stats, counters, 2 * sizeof(unsigned int), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "tc stats copy");
    }
    return CKM_OK;
}

}  // namespace ckm
