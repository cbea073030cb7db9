// Any-shape Lloyd kernels (any d, any k; FP32 and FP64 point types) and the
// small helper kernels of the three-stage path.
//
// The generic kernel is one thread per point (grid-stride).  Centroids live
// in shared memory when they fit, else they are read through L1.  Per-point
// arithmetic is the reference's (kmeans_naive.cpp:48-63; for double the FP64
// path of KmeansNaive64).  Sums go to a per-CTA shared-memory table when it
// fits (merged once into FP64 scratch) or straight into the FP64 scratch with
// global atomics.  Like the low-d kernel, the last CTA finalises.
#include "ckm_device.cuh"
#include "ckm_internal.h"
#include "ckm_mma_screen.cuh"

#include <algorithm>
#include <cstdlib>
#include <mutex>

namespace ckm {
namespace {

constexpr int GBLK = 256;
constexpr size_t GENERIC_SMEM_LIMIT = 96 * 1024;

template <typename T, typename L, typename M>
struct GenericArgs {
    const T* points;
    const T* centroids;
    L* labels;
    T* new_centroids;
    M* masses;
    ScratchView scratch;
    uint64_t n;
    uint32_t d, k;
    int mode;
};

// Shared-memory accumulator element type: FP32 points sum in FP32 per CTA
// (merged into FP64 once); FP64 points sum in FP64.
template <typename T> struct AccT { using type = T; };

template <typename T, typename L, typename M, Pass PASS>
__global__ void __launch_bounds__(GBLK)
    generic_kernel(const GenericArgs<T, L, M> a, const int cent_smem, const int acc_smem) {
    extern __shared__ __align__(16) unsigned char smem[];
    using A = typename AccT<T>::type;
    const uint32_t k = a.k, d = a.d;
    const uint64_t n = a.n;
    const uint64_t kd = (uint64_t)k * d;

    T* s_c = reinterpret_cast<T*>(smem);                    // [c * d + f]
    size_t off = cent_smem ? ((kd * sizeof(T) + 15) & ~size_t(15)) : 0;
    A* s_sum = reinterpret_cast<A*>(smem + off);            // [f * k + c]
    unsigned int* s_mass = reinterpret_cast<unsigned int*>(smem + off + ((kd * sizeof(A) + 15) & ~size_t(15)));

    if (PASS != Pass::SumsOnly && cent_smem) {
        for (uint64_t i = threadIdx.x; i < kd; i += GBLK) {
            const uint64_t c = i / d, f = i - c * d;
            s_c[i] = a.centroids[f * k + c];
        }
    }
    if (PASS != Pass::LabelOnly && acc_smem) {
        for (uint64_t i = threadIdx.x; i < kd; i += GBLK) s_sum[i] = A(0);
        for (uint32_t i = threadIdx.x; i < k; i += GBLK) s_mass[i] = 0u;
    }
    __syncthreads();

    for (uint64_t p = (uint64_t)blockIdx.x * GBLK + threadIdx.x; p < n; p += (uint64_t)gridDim.x * GBLK) {
        uint64_t lab;
        if constexpr (PASS == Pass::SumsOnly) {
            lab = (uint64_t)a.labels[p];
        } else {
            T best = TypeMax<T>::v();
            lab = 0;
            for (uint32_t c = 0; c < k; ++c) {
                T dist = T(0);
                if (cent_smem) {
                    const T* cr = s_c + (uint64_t)c * d;
                    for (uint32_t f = 0; f < d; ++f) {
                        const T t = __ldg(a.points + (uint64_t)f * n + p) - cr[f];
                        dist = fma(t, t, dist);
                    }
                } else {
                    for (uint32_t f = 0; f < d; ++f) {
                        const T t = __ldg(a.points + (uint64_t)f * n + p) - __ldg(a.centroids + (uint64_t)f * k + c);
                        dist = fma(t, t, dist);
                    }
                }
                if (dist < best) {
                    best = dist;
                    lab = c;
                }
            }
            a.labels[p] = (L)lab;
        }
        if constexpr (PASS != Pass::LabelOnly) {
            if (lab < k) {
                if (acc_smem) {
                    for (uint32_t f = 0; f < d; ++f)
                        atomicAdd(&s_sum[(uint64_t)f * k + lab], (A)__ldg(a.points + (uint64_t)f * n + p));
                    atomicAdd(&s_mass[lab], 1u);
                } else {
                    for (uint32_t f = 0; f < d; ++f)
                        atomicAdd(&a.scratch.sums[(uint64_t)f * k + lab], (double)__ldg(a.points + (uint64_t)f * n + p));
                    atomicAdd(&a.scratch.masses[lab], 1ull);
                }
            }
        }
    }

    if constexpr (PASS == Pass::LabelOnly) {
        return;
    } else {
        if (acc_smem) {
            __syncthreads();
            for (uint64_t i = threadIdx.x; i < kd; i += GBLK) {
                const A v = s_sum[i];
                if (v != A(0)) atomicAdd(&a.scratch.sums[i], (double)v);
            }
            for (uint32_t i = threadIdx.x; i < k; i += GBLK) {
                const unsigned int v = s_mass[i];
                if (v) atomicAdd(&a.scratch.masses[i], (unsigned long long)v);
            }
        }
        if (a.mode == CKM_MODE_DEFER) return;
        if (last_cta_ticket(a.scratch.ctrl)) finalize_block<T, M>(d, k, a.new_centroids, a.masses, a.scratch, a.mode);
    }
}

template <typename T, typename L, typename M>
int launch_generic_t(const GenericArgs<T, L, M>& a, Pass pass, cudaStream_t s) {
    const DeviceInfo& di = device_info();
    const uint64_t kd = (uint64_t)a.k * a.d;
    const size_t cent_bytes = (kd * sizeof(T) + 15) & ~size_t(15);
    const size_t acc_bytes = ((kd * sizeof(T) + 15) & ~size_t(15)) + (((size_t)a.k * 4 + 15) & ~size_t(15));
    int cent_smem = (pass != Pass::SumsOnly) && cent_bytes <= GENERIC_SMEM_LIMIT / 2;
    int acc_smem = (pass != Pass::LabelOnly) && acc_bytes <= GENERIC_SMEM_LIMIT / 2;
    size_t smem = (cent_smem ? cent_bytes : 0) + (acc_smem ? acc_bytes : 0);

    void (*kern)(const GenericArgs<T, L, M>, const int, const int) = nullptr;
    switch (pass) {
        case Pass::Fused: kern = generic_kernel<T, L, M, Pass::Fused>; break;
        case Pass::LabelOnly: kern = generic_kernel<T, L, M, Pass::LabelOnly>; break;
        case Pass::SumsOnly: kern = generic_kernel<T, L, M, Pass::SumsOnly>; break;
    }
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> g(mu);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GENERIC_SMEM_LIMIT);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(generic)");
    }
    int bps = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, GBLK, smem);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy(generic)");
    if (bps < 1) bps = 1;
    uint64_t blocks = (a.n + GBLK - 1) / GBLK;
    uint64_t grid = std::min<uint64_t>(blocks, (uint64_t)di.sm_count * bps);
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, GBLK, smem, s>>>(a, cent_smem, acc_smem);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "generic launch");
    return CKM_OK;
}

// ---------------------------------------------------------------------------
// Fixed-d FP32 kernel for mid-size d (32, 64).  Each thread loads its point
// once into registers (one coalesced load per feature), labels it against the
// centroid rows in shared memory with label_rows_exact (four independent
// cluster chains, 128-bit row loads) and adds the registers into the CTA's
// shared-memory table, merged once into the FP64 scratch.  The generic kernel
// re-reads the point for every cluster and runs one dependent fma chain at a
// time; the outputs are the same.  Labels come from a certified screen, the
// tensor-core one (mma_label8) for d = 32 with k >= 64 and d = 64 with
// k >= 32 where its TF32 fragments fit in shared memory, else the FP32 one
// (label_rows_screened); both fall back to exact arithmetic per point.
// ---------------------------------------------------------------------------

// label_mode: 0 exact loop, 1 FP32 screen (label_rows_screened), 2 tensor-core
// screen (mma_label8: 8 points per warp; centroids staged as TF32 fragments).
template <int D, Pass PASS, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    rows_kernel(const GenericArgs<float, uint32_t, uint32_t> a, const uint32_t copies, const int label_mode) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t k = a.k;
    const uint64_t n = a.n;
    const uint32_t kd = k * D;
    const bool mma = label_mode == 2;
    // `copies` (a power of two up to 32) interleaved copies of the sums,
    // s_sum[(f * k + c) * copies + (lane & (copies - 1))]: a shared-memory
    // FP32 atomic add retries while other lanes of the warp hit the same word,
    // and the copies keep the lanes apart (with 32 they never meet).  Masses
    // (integer atomics, which do not slow down that way) keep one copy.
    const uint32_t lane_off = threadIdx.x & (copies - 1u);
    __shared__ unsigned int s_cn_max;
    float* s_c = reinterpret_cast<float*>(smem);  // rows [c * D + f], or the MMA fragments
    float* s_cn = mma ? s_c + (size_t)mma_k_pad(k) * D * 2 : s_c + kd;  // |c|^2 for the screens
    float* s_sum = mma ? reinterpret_cast<float*>(smem + mma_cent_bytes(k, D)) : s_cn + ((k + 3u) & ~3u);
    unsigned int* s_mass = reinterpret_cast<unsigned int*>(s_sum + (size_t)kd * copies);

    if (threadIdx.x == 0) s_cn_max = 0u;
    if constexpr (PASS == Pass::Fused) {
        const size_t words = (size_t)kd * copies + k;
        for (size_t i = threadIdx.x; i < words; i += NT) s_sum[i] = 0.0f;  // sums, then masses
    }
    if (mma) {
        __syncthreads();  // s_cn_max is zero before the staging's atomicMax
        mma_stage_centroids<D>(a.centroids, k, reinterpret_cast<float4*>(s_c), s_cn, &s_cn_max, threadIdx.x, NT);
        __syncthreads();
    } else {
        for (uint32_t i = threadIdx.x; i < kd; i += NT) {
            const uint32_t c = i / D, f = i - c * D;
            s_c[i] = a.centroids[(size_t)f * k + c];
        }
        __syncthreads();
        if (label_mode == 1) {
            screen_norms(s_c, D, k, s_cn, &s_cn_max, threadIdx.x, NT);
            __syncthreads();
        }
    }
    const float cm = screen_cm(s_cn_max);

    if (mma) {
        // 8 points per warp iteration; each lane adds its quarter of its
        // point's features (x = hi + mid exactly)
        const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, g = lane >> 2, t = lane & 3u;
        const uint64_t stride = (uint64_t)gridDim.x * (NT / 32) * 8;
#pragma unroll 1
        for (uint64_t p0 = ((uint64_t)blockIdx.x * (NT / 32) + warp) * 8; p0 < n; p0 += stride) {
            uint32_t bh[D / 4], bm[D / 4];
            uint32_t lab;
            mma_label8<D>(a.points, n, p0, n, reinterpret_cast<const float4*>(s_c), s_cn, cm, k, bh, bm, lab);
            if (p0 + g < n) {
                if (t == 0) a.labels[p0 + g] = lab;
                if constexpr (PASS == Pass::Fused) {
#pragma unroll
                    for (uint32_t i = 0; i < (uint32_t)D / 4; ++i) {
                        const uint32_t f = (i >> 1) * 8 + t + ((i & 1u) ? 4u : 0u);
                        atomicAdd(&s_sum[((size_t)f * k + lab) * copies + lane_off],
                                  __uint_as_float(bh[i]) + __uint_as_float(bm[i]));
                    }
                    if (t == 0) atomicAdd(&s_mass[lab], 1u);
                }
            }
        }
    } else {
        for (uint64_t p = (uint64_t)blockIdx.x * NT + threadIdx.x; p < n; p += (uint64_t)gridDim.x * NT) {
            float x[D];
#pragma unroll
            for (int f = 0; f < D; ++f) x[f] = __ldg(a.points + (uint64_t)f * n + p);
            const uint32_t lab =
                label_mode == 1 ? label_rows_screened<D>(x, s_c, s_cn, cm, k) : label_rows_exact<D>(x, s_c, k);
            a.labels[p] = lab;
            if constexpr (PASS == Pass::Fused) {
#pragma unroll
                for (int f = 0; f < D; ++f) atomicAdd(&s_sum[((size_t)f * k + lab) * copies + lane_off], x[f]);
                atomicAdd(&s_mass[lab], 1u);
            }
        }
    }

    if constexpr (PASS == Pass::Fused) {
        __syncthreads();
        if (copies == 32) {
            const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            for (uint32_t e = warp; e < kd; e += NT / 32) {
                const float v = warp_sum_f32(s_sum[(size_t)e * 32 + lane]);
                if (lane == 0 && v != 0.0f) atomicAdd(&a.scratch.sums[e], (double)v);
            }
        } else {
            for (uint32_t e = threadIdx.x; e < kd; e += NT) {
                float v = 0.0f;
                for (uint32_t j = 0; j < copies; ++j) v += s_sum[(size_t)e * copies + j];
                if (v != 0.0f) atomicAdd(&a.scratch.sums[e], (double)v);
            }
        }
        for (uint32_t i = threadIdx.x; i < k; i += NT) {
            const unsigned int v = s_mass[i];
            if (v) atomicAdd(&a.scratch.masses[i], (unsigned long long)v);
        }
        if (a.mode == CKM_MODE_DEFER) return;
        if (last_cta_ticket(a.scratch.ctrl)) finalize_block<float, uint32_t>(D, k, a.new_centroids, a.masses, a.scratch, a.mode);
    }
}

size_t rows_smem_bytes(uint32_t d, uint32_t k, Pass pass, uint32_t copies, bool mma) {
    const size_t kd = (size_t)k * d;
    const size_t cent = mma ? mma_cent_bytes(k, d) : (kd + ((k + 3) & ~size_t(3))) * sizeof(float);  // + |c|^2
    return cent + (pass == Pass::Fused ? (kd * copies + k) * sizeof(float) : 0);
}

// The labelling of the rows kernel: the environment variable CKM_SCREEN = "0"
// selects the exact loop for every cluster, "1" the FP32 screen for every
// shape; otherwise the tensor-core screen where mma_min_k allows, else the
// FP32 screen.
int screen_setting() {
    static int v = [] {
        const char* e = getenv("CKM_SCREEN");
        return (e && (e[0] == '0' || e[0] == '1')) ? e[0] - '0' : 2;
    }();
    return v;
}

constexpr size_t ROWS_TWO_CTA_LIMIT = 110 * 1024;  // two 256-thread CTAs per SM
constexpr size_t ROWS_COPIES_LIMIT = 200 * 1024;  // tables of several copies up to this size

template <int D, Pass PASS, int NT, int MINB>
int launch_rows_v(const GenericArgs<float, uint32_t, uint32_t>& a, size_t smem, uint32_t copies, int label_mode,
                  cudaStream_t s) {
    auto kern = rows_kernel<D, PASS, NT, MINB>;
    static std::mutex mu;
    static bool attr_done[64] = {false};
    const DeviceInfo& di = device_info();
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> g(mu);
        if (dev < 0 || dev >= 64 || !attr_done[dev]) {
            cudaFuncAttributes fa;
            cudaError_t e = cudaFuncGetAttributes(&fa, kern);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(rows)");
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(di.smem_optin - fa.sharedSizeBytes));
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rows)");
            if (dev >= 0 && dev < 64) attr_done[dev] = true;
        }
    }
    int bps = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, NT, smem);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy(rows)");
    if (bps < 1) return fail(CKM_ERR_UNSUPPORTED, "rows: kernel does not fit on an SM");
    const uint64_t per_cta = label_mode == 2 ? (uint64_t)(NT / 32) * 8 : (uint64_t)NT;
    const uint64_t blocks = (a.n + per_cta - 1) / per_cta;
    uint64_t grid = std::min<uint64_t>(blocks, (uint64_t)di.sm_count * bps);
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, NT, smem, s>>>(a, copies, label_mode);
    count_launch();
    e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "rows launch");
}

template <int D, Pass PASS>
int launch_rows_d(const GenericArgs<float, uint32_t, uint32_t>& a, cudaStream_t s) {
    const int setting = screen_setting();
    bool mma = setting == 2 && a.k >= mma_min_k(D) &&
               rows_smem_bytes(D, a.k, PASS, 1, true) + 1024 <= device_info().smem_optin;
    const int label_mode = mma ? 2 : (setting == 0 ? 0 : 1);
    // the most copies that keep the table within the limit (one at least)
    uint32_t copies = 1;
    if (PASS == Pass::Fused)
        for (uint32_t c = 32; c > 1; c >>= 1)
            if (rows_smem_bytes(D, a.k, PASS, c, mma) <= ROWS_COPIES_LIMIT) {
                copies = c;
                break;
            }
    const size_t smem = rows_smem_bytes(D, a.k, PASS, copies, mma);
    if (smem <= ROWS_TWO_CTA_LIMIT) return launch_rows_v<D, PASS, 256, 2>(a, smem, copies, label_mode, s);
    return launch_rows_v<D, PASS, 512, 1>(a, smem, copies, label_mode, s);
}

// Returns -1000 when the shape is not one the rows kernel takes.
int try_launch_rows(const GenericArgs<float, uint32_t, uint32_t>& a, Pass pass, cudaStream_t s) {
    if (pass == Pass::SumsOnly || (a.d != 32 && a.d != 64)) return -1000;
    if (rows_smem_bytes(a.d, a.k, pass, 1, false) + 1024 > device_info().smem_optin) return -1000;
    if (pass == Pass::Fused) return a.d == 32 ? launch_rows_d<32, Pass::Fused>(a, s) : launch_rows_d<64, Pass::Fused>(a, s);
    return a.d == 32 ? launch_rows_d<32, Pass::LabelOnly>(a, s) : launch_rows_d<64, Pass::LabelOnly>(a, s);
}

// ---------------------------------------------------------------------------
// Helper kernels.
// ---------------------------------------------------------------------------
template <typename T, typename M>
__global__ void finalize_kernel(uint32_t d, uint32_t k, T* C, M* masses, ScratchView sv, int mode) {
    finalize_block<T, M>(d, k, C, masses, sv, mode);
}

// Label histogram (exact): per-CTA shared-memory bins, one global add per
// non-empty bin.  Labels outside [0, k) are ignored.
template <typename L, typename M>
__global__ void __launch_bounds__(256) mass_kernel(const L* __restrict__ labels, uint64_t n, uint32_t k,
                                                   M* __restrict__ masses, int bins_smem) {
    extern __shared__ unsigned int s_bins[];
    if (bins_smem) {
        for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) s_bins[i] = 0u;
        __syncthreads();
    }
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t l = (uint64_t)labels[p];
        if (l < k) {
            if (bins_smem) atomicAdd(&s_bins[l], 1u);
            else atomicAdd(&masses[l], (M)1);
        }
    }
    if (bins_smem) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < k; i += blockDim.x)
            if (s_bins[i]) atomicAdd(&masses[i], (M)s_bins[i]);
    }
}

template <typename T, typename M>
__global__ void divide_kernel(uint32_t d, uint32_t k, T* m, const M* masses) {
    const uint64_t kd = (uint64_t)k * d;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kd; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(i % k);
        m[i] = m[i] / (T)masses[c];
    }
}

template <typename T>
__global__ void add_kernel(uint64_t count, T* a, const T* b) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x)
        a[i] = a[i] + b[i];
}

// Column sums of a column-major rows x cols uint32 matrix into data[0..rows).
// Element (row, 0) is read only by the thread(s) that own `row`, so the
// in-place write is safe.
__global__ void reduce_parcol_rows_kernel(uint64_t cols, uint64_t rows, uint32_t* data) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = 0;
        for (uint64_t c = 0; c < cols; ++c) s += data[c * rows + r];
        data[r] = s;
    }
}

__global__ void reduce_parcol_block_kernel(uint64_t cols, uint64_t rows, uint32_t* data) {
    __shared__ uint32_t part[32];
    const uint64_t r = blockIdx.x;
    uint32_t s = 0;
    for (uint64_t c = threadIdx.x; c < cols; c += blockDim.x) s += data[c * rows + r];
    s = __reduce_add_sync(0xffffffffu, s);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0u;
        v = __reduce_add_sync(0xffffffffu, v);
        if (threadIdx.x == 0) data[r] = v;
    }
}

// --- Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011), the published counter-based generator.
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 philox(U4 ctr, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * ctr.x, hi0 = __umulhi(0xD2511F53u, ctr.x);
        const uint32_t lo1 = 0xCD9E8D57u * ctr.z, hi1 = __umulhi(0xCD9E8D57u, ctr.z);
        ctr = U4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ctr;
}
__device__ __forceinline__ float u01(uint32_t v) {  // (0, 1]
    return ((float)(v >> 8) + 1.0f) * (1.0f / 16777216.0f);
}

// Blob b: centre_f = lo + (hi - lo) * U, sigma = slo + (shi - slo) * U.
// Point p: blob = floor(U * blobs); x_f = centre_f + sigma * N(0, 1), the
// normals by Box-Muller from one Philox block per 4 features.
__global__ void __launch_bounds__(256) generate_kernel(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed,
                                                       float clo, float chi, float slo, float shi,
                                                       uint64_t first, float* out, uint64_t stride) {
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = first + i;
        const U4 sel = philox(U4{(uint32_t)p, (uint32_t)(p >> 32), 0xB10Bu, 0u}, k0, k1);
        const uint32_t b = (uint32_t)(((uint64_t)sel.x * blobs) >> 32);
        const U4 sg = philox(U4{b, 0u, 0x516Au, 1u}, k0, k1);
        const float sigma = slo + (shi - slo) * (u01(sg.x) - (1.0f / 16777216.0f));
        for (uint32_t f0 = 0; f0 < d; f0 += 4) {
            const U4 r = philox(U4{(uint32_t)p, (uint32_t)(p >> 32), 0xD47Au + f0, 2u}, k0, k1);
            float z[4];
            {
                const float rad = sqrtf(-2.0f * logf(u01(r.x)));
                float sn, cs;
                sincospif(2.0f * u01(r.y), &sn, &cs);
                z[0] = rad * cs; z[1] = rad * sn;
            }
            {
                const float rad = sqrtf(-2.0f * logf(u01(r.z)));
                float sn, cs;
                sincospif(2.0f * u01(r.w), &sn, &cs);
                z[2] = rad * cs; z[3] = rad * sn;
            }
            for (uint32_t j = 0; j < 4 && f0 + j < d; ++j) {
                const uint32_t f = f0 + j;
                const U4 cc = philox(U4{b, f, 0xCE47u, 3u}, k0, k1);
                const float centre = clo + (chi - clo) * (u01(cc.x) - (1.0f / 16777216.0f));
                out[(uint64_t)f * stride + i] = centre + sigma * z[j];
            }
        }
    }
}

__device__ __forceinline__ float normal01(uint32_t a, uint32_t b, int which) {
    const float rad = sqrtf(-2.0f * logf(u01(a)));
    float sn, cs;
    sincospif(2.0f * u01(b), &sn, &cs);
    return rad * (which ? sn : cs);
}

// Mixture with a chosen centre law (uniform in [a, b] or normal with mean a
// and standard deviation b), sigma law (uniform or log-uniform in [lo, hi])
// and component weights (equal, or Dirichlet(1): normalised Exp(1) draws).
// The weights' cumulative table is rebuilt in shared memory by every CTA.
__global__ void __launch_bounds__(256) generate_ex_kernel(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed,
                                                          int center_dist, float ca, float cb, int sigma_dist,
                                                          float slo, float shi, int dirichlet, uint64_t first,
                                                          float* out, uint64_t stride) {
    extern __shared__ float s_cdf[];
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    if (dirichlet) {
        for (uint32_t b = threadIdx.x; b < blobs; b += blockDim.x) {
            const U4 r = philox(U4{b, 0u, 0xD1A1u, 4u}, k0, k1);
            s_cdf[b] = -logf(u01(r.x));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float acc = 0.f;
            for (uint32_t b = 0; b < blobs; ++b) {
                acc += s_cdf[b];
                s_cdf[b] = acc;
            }
        }
        __syncthreads();
    }
    const float total = dirichlet ? s_cdf[blobs - 1] : 1.0f;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p = first + i;
        const U4 sel = philox(U4{(uint32_t)p, (uint32_t)(p >> 32), 0xB10Bu, 0u}, k0, k1);
        uint32_t b;
        if (dirichlet) {
            const float u = u01(sel.x) * total;
            uint32_t lo = 0, hi = blobs - 1;
            while (lo < hi) {  // first b with cdf[b] >= u
                const uint32_t mid = (lo + hi) >> 1;
                if (s_cdf[mid] >= u) hi = mid;
                else lo = mid + 1;
            }
            b = lo;
        } else {
            b = (uint32_t)(((uint64_t)sel.x * blobs) >> 32);
        }
        const U4 sg = philox(U4{b, 0u, 0x516Au, 1u}, k0, k1);
        const float us = u01(sg.x) - (1.0f / 16777216.0f);
        const float sigma = sigma_dist ? expf(logf(slo) + (logf(shi) - logf(slo)) * us) : slo + (shi - slo) * us;
        for (uint32_t f0 = 0; f0 < d; f0 += 4) {
            const U4 r = philox(U4{(uint32_t)p, (uint32_t)(p >> 32), 0xD47Au + f0, 2u}, k0, k1);
            const float z[4] = {normal01(r.x, r.y, 0), normal01(r.x, r.y, 1), normal01(r.z, r.w, 0),
                                normal01(r.z, r.w, 1)};
            for (uint32_t j = 0; j < 4 && f0 + j < d; ++j) {
                const uint32_t f = f0 + j;
                const U4 cc = philox(U4{b, f, 0xCE47u, 3u}, k0, k1);
                const float centre = center_dist ? ca + cb * normal01(cc.x, cc.y, 0)
                                                 : ca + (cb - ca) * (u01(cc.x) - (1.0f / 16777216.0f));
                out[(uint64_t)f * stride + i] = centre + sigma * z[j];
            }
        }
    }
}

int grid_for(uint64_t work, int block) {
    uint64_t g = (work + block - 1) / block;
    const uint64_t cap = (uint64_t)device_info().sm_count * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

int launch_generic_f32(const FusedF32& a, Pass pass, cudaStream_t s) {
    GenericArgs<float, uint32_t, uint32_t> g{a.points, a.centroids, a.labels, a.new_centroids, a.masses,
                                             a.scratch, a.n, a.d, a.k, a.mode};
    const int st = try_launch_rows(g, pass, s);
    if (st != -1000) return st;
    return launch_generic_t(g, pass, s);
}

int launch_generic_f64(const FusedF64& a, Pass pass, cudaStream_t s) {
    GenericArgs<double, uint64_t, uint64_t> g{a.points, a.centroids, a.labels, a.new_centroids, a.masses,
                                              a.scratch, a.n, a.d, a.k, a.mode};
    return launch_generic_t(g, pass, s);
}

int launch_finalize_f32(uint32_t d, uint32_t k, float* c, uint32_t* m, ScratchView sv, int mode, cudaStream_t s) {
    finalize_kernel<float, uint32_t><<<1, 1024, 0, s>>>(d, k, c, m, sv, mode);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "finalize launch");
}

int launch_finalize_f64(uint32_t d, uint32_t k, double* c, uint64_t* m, ScratchView sv, int mode, cudaStream_t s) {
    finalize_kernel<double, uint64_t><<<1, 1024, 0, s>>>(d, k, c, m, sv, mode);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "finalize launch");
}

template <typename L, typename M>
static int launch_mass_t(uint64_t n, uint32_t k, const L* labels, M* masses, cudaStream_t s) {
    const int bins_smem = (size_t)k * 4 <= 48 * 1024;
    const size_t smem = bins_smem ? (size_t)k * 4 : 0;
    mass_kernel<L, M><<<grid_for(n, 256), 256, smem, s>>>(labels, n, k, masses, bins_smem);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "mass launch");
}

int launch_mass_u32(uint64_t n, uint32_t k, const uint32_t* labels, uint32_t* masses, cudaStream_t s) {
    return launch_mass_t<uint32_t, unsigned int>(n, k, labels, reinterpret_cast<unsigned int*>(masses), s);
}

int launch_mass_u64(uint64_t n, uint32_t k, const uint64_t* labels, uint64_t* masses, cudaStream_t s) {
    return launch_mass_t<uint64_t, unsigned long long>(n, k, labels, reinterpret_cast<unsigned long long*>(masses), s);
}

// Relative centroid shift: max |new - old| over max |old| (NaN entries, the
// empty clusters, are skipped by fmaxf).  One CTA.
template <typename T>
__global__ void __launch_bounds__(1024) shift_kernel(uint64_t kd, const T* __restrict__ old_c,
                                                     const T* __restrict__ new_c, float* __restrict__ out) {
    __shared__ float s_a[32], s_b[32];
    float a = 0.0f, b = 0.0f;
    for (uint64_t e = threadIdx.x; e < kd; e += blockDim.x) {
        const T o = old_c[e];
        a = fmaxf(a, (float)fabs((double)new_c[e] - (double)o));
        b = fmaxf(b, (float)fabs((double)o));
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_a[threadIdx.x >> 5] = a;
        s_b[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 1; w < blockDim.x / 32; ++w) {
            a = fmaxf(a, s_a[w]);
            b = fmaxf(b, s_b[w]);
        }
        out[0] = a / fmaxf(b, 1e-30f);
    }
}

int launch_shift_f32(uint64_t kd, const float* o, const float* n, float* out, cudaStream_t s) {
    shift_kernel<float><<<1, 1024, 0, s>>>(kd, o, n, out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "shift launch");
}

int launch_shift_f64(uint64_t kd, const double* o, const double* n, float* out, cudaStream_t s) {
    shift_kernel<double><<<1, 1024, 0, s>>>(kd, o, n, out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "shift launch");
}

int launch_divide_f32(uint32_t d, uint32_t k, float* m, const uint32_t* masses, cudaStream_t s) {
    divide_kernel<float, uint32_t><<<grid_for((uint64_t)k * d, 256), 256, 0, s>>>(d, k, m, masses);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "divide launch");
}

int launch_divide_f64(uint32_t d, uint32_t k, double* m, const uint64_t* masses, cudaStream_t s) {
    divide_kernel<double, uint64_t><<<grid_for((uint64_t)k * d, 256), 256, 0, s>>>(d, k, m, masses);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "divide launch");
}

template <typename T>
int launch_add(uint64_t count, T* a, const T* b, cudaStream_t s) {
    add_kernel<T><<<grid_for(count, 256), 256, 0, s>>>(count, a, b);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "add launch");
}
template int launch_add<float>(uint64_t, float*, const float*, cudaStream_t);
template int launch_add<double>(uint64_t, double*, const double*, cudaStream_t);
template int launch_add<uint32_t>(uint64_t, uint32_t*, const uint32_t*, cudaStream_t);
template int launch_add<uint64_t>(uint64_t, uint64_t*, const uint64_t*, cudaStream_t);

int launch_reduce_parcol_u32(uint64_t cols, uint64_t rows, uint32_t* data, cudaStream_t s) {
    if (rows >= 128) reduce_parcol_rows_kernel<<<grid_for(rows, 128), 128, 0, s>>>(cols, rows, data);
    else reduce_parcol_block_kernel<<<(unsigned)rows, 256, 0, s>>>(cols, rows, data);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "reduce_vector_parcol launch");
}

int launch_generate_f32(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed, float clo, float chi, float slo,
                        float shi, uint64_t first, float* out, uint64_t stride, cudaStream_t s) {
    generate_kernel<<<grid_for(n, 256), 256, 0, s>>>(d, n, blobs, seed, clo, chi, slo, shi, first, out, stride);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "generate launch");
}

int launch_generate_ex_f32(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed, int center_dist, float ca,
                           float cb, int sigma_dist, float slo, float shi, int dirichlet, uint64_t first, float* out,
                           uint64_t stride, cudaStream_t s) {
    const size_t smem = dirichlet ? (size_t)blobs * sizeof(float) : 0;
    if (smem > 48 * 1024) return fail(CKM_ERR_UNSUPPORTED, "Dirichlet weights: at most 12288 blobs");
    generate_ex_kernel<<<grid_for(n, 256), 256, smem, s>>>(d, n, blobs, seed, center_dist, ca, cb, sigma_dist, slo,
                                                          shi, dirichlet, first, out, stride);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "generate launch");
}

}  // namespace ckm
