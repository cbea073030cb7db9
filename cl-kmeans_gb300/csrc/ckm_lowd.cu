// Low-dimensional Lloyd kernels (d <= 16), FP32.
//
// One persistent launch per pass.  Each CTA (256 threads) keeps the centroids
// in shared memory as duplicated (c, c) pairs, streams column-major points in
// 128-bit loads (P[f * n + p], lloyd_fused_feature_sum.cl:200), two tiles in
// flight per thread, and for each thread's points:
//   - labels them with the reference's exact arithmetic
//     (t = x_f - c_f; acc = fma(t, t, acc); strict '<' argmin from c = 0,
//      lloyd_fused_feature_sum.cl:213-239), two points per packed FP32x2 op;
//   - adds the point into a shared-memory partial table.  For small k*(d+1)
//     every thread owns a private column of the table (no atomics, no bank
//     conflicts); otherwise the 32 lanes own columns shared by the CTA's warps
//     (shared-memory atomics);
//   - at the end merges its table once into FP64 scratch (warp tree in FP32,
//     FP64 atomics), which replaces the reference's global partials,
//     ReduceVectorParcol and MatrixBinaryOp::matrix add
//     (fused_feature_sum.hpp:224-439);
//   - the last CTA to finish divides sums by masses
//     (MatrixBinaryOp::row divide, matrix_binary_op.cl:98-114) and re-zeroes
//     the scratch, so a whole Lloyd iteration is one launch.
#include "ckm_device.cuh"
#include "ckm_internal.h"

#include <cstdlib>
#include <mutex>
#include <unordered_map>

namespace ckm {
namespace {

constexpr int BLK = 256;

template <int D> struct LowdCfg {
    static constexpr int PPT = D <= 4 ? 8 : (D <= 8 ? 4 : 2);  // points per thread per tile
    static constexpr int VW = PPT < 4 ? PPT : 4;                 // floats per vector load
};

template <int D> struct AccVec {
    static constexpr int VG = (D % 4 == 0) ? 4 : ((D % 2 == 0) ? 2 : 1);  // floats per table vector
};

template <int D, int PPT>
struct Tile {
    float x[D][PPT];
    uint32_t lab[PPT];
};

template <int VW>
__device__ __forceinline__ void load_vec(float* dst, const float* src) {
    if constexpr (VW == 4) {
        float4 v = __ldg(reinterpret_cast<const float4*>(src));
        dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; dst[3] = v.w;
    } else if constexpr (VW == 2) {
        float2 v = __ldg(reinterpret_cast<const float2*>(src));
        dst[0] = v.x; dst[1] = v.y;
    } else {
        dst[0] = __ldg(src);
    }
}

template <int D, int PPT, Pass PASS>
__device__ __forceinline__ void load_tile(Tile<D, PPT>& T, const FusedF32& a, uint64_t p0, bool vec) {
    constexpr int VW = LowdCfg<D>::VW;
    const uint64_t n = a.n;
    if (vec && p0 + PPT <= n) {
#pragma unroll
        for (int f = 0; f < D; ++f)
#pragma unroll
            for (int v = 0; v < PPT; v += VW) load_vec<VW>(&T.x[f][v], a.points + (uint64_t)f * n + p0 + v);
        if constexpr (PASS == Pass::SumsOnly) {
#pragma unroll
            for (int v = 0; v < PPT; v += VW) {
                if constexpr (VW == 4) {
                    uint4 l = __ldg(reinterpret_cast<const uint4*>(a.labels + p0 + v));
                    T.lab[v] = l.x; T.lab[v + 1] = l.y; T.lab[v + 2] = l.z; T.lab[v + 3] = l.w;
                } else if constexpr (VW == 2) {
                    uint2 l = __ldg(reinterpret_cast<const uint2*>(a.labels + p0 + v));
                    T.lab[v] = l.x; T.lab[v + 1] = l.y;
                } else {
                    T.lab[v] = __ldg(a.labels + p0 + v);
                }
            }
        }
    } else {
#pragma unroll
        for (int i = 0; i < PPT; ++i) {
            const bool ok = p0 + i < n;
#pragma unroll
            for (int f = 0; f < D; ++f) T.x[f][i] = ok ? __ldg(a.points + (uint64_t)f * n + p0 + i) : 0.0f;
            if constexpr (PASS == Pass::SumsOnly) T.lab[i] = ok ? __ldg(a.labels + p0 + i) : 0xffffffffu;
        }
    }
}

// Order-preserving map of floats to unsigned integers (and back), so warp
// minima / maxima of floats run as one integer reduction.
__device__ __forceinline__ uint32_t f2o(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Box pruning (k <= 32): the clusters that can hold the reference's label of
// some point of this warp.  The warp's points lie in the box [lo, hi]
// (per-feature minima and maxima; NaN coordinates are left out: a point with
// a NaN has NaN distances everywhere and label 0 whatever is pruned).  For
// cluster c, LB_c = sum_f max(lo_f - c_f, c_f - hi_f, 0)^2 (rounded down) is
// at most its squared distance to any point of the box, UB_c =
// sum_f max(|c_f - lo_f|, |c_f - hi_f|)^2 (rounded up) at least.  With the
// reference's FP32 distance within (1 +- rho) of the exact one,
// rho = (D + 4) 2^-24, a cluster with LB_c (1 - rho) > min UB (1 + rho) +
// 2^-120 (underflow) is farther, in the reference's arithmetic, than the
// cluster of min UB from every point of the box: it can neither be the
// label nor tie it.  The mask is the same in every lane.
template <int D, int PPT>
__device__ __forceinline__ uint32_t box_prune_mask(const Tile<D, PPT>& T, uint64_t p0, uint64_t n,
                                                   const float2* __restrict__ s_c, uint32_t k) {
    const uint32_t lane = threadIdx.x & 31u;
    float lo[D], hi[D];
#pragma unroll
    for (int f = 0; f < D; ++f) {
        lo[f] = INFINITY;
        hi[f] = -INFINITY;
    }
#pragma unroll
    for (int i = 0; i < PPT; ++i)
        if (p0 + i < n) {
#pragma unroll
            for (int f = 0; f < D; ++f) {
                lo[f] = fminf(lo[f], T.x[f][i]);
                hi[f] = fmaxf(hi[f], T.x[f][i]);
            }
        }
#pragma unroll
    for (int f = 0; f < D; ++f) {
        lo[f] = o2f(__reduce_min_sync(0xffffffffu, f2o(lo[f])));
        hi[f] = o2f(__reduce_max_sync(0xffffffffu, f2o(hi[f])));
    }
    float lb = INFINITY, ub = INFINITY;
    if (lane < k) {
        lb = 0.0f;
        ub = 0.0f;
#pragma unroll
        for (int f = 0; f < D; ++f) {
            const float c = s_c[lane * D + f].x;
            const float g = fmaxf(fmaxf(__fsub_rd(lo[f], c), __fsub_rd(c, hi[f])), 0.0f);
            lb = __fmaf_rd(g, g, lb);
            const float u = fmaxf(fmaxf(__fsub_ru(c, lo[f]), __fsub_ru(lo[f], c)),
                                  fmaxf(__fsub_ru(c, hi[f]), __fsub_ru(hi[f], c)));
            ub = __fmaf_ru(u, u, ub);
        }
        if (isnan(ub)) ub = INFINITY;
    }
    const float ub_min = o2f(__reduce_min_sync(0xffffffffu, f2o(ub)));
    constexpr float kLo = 1.0f - (float)(D + 4) * 0x1p-24f;       // exact
    constexpr float kHi = 1.0f + (float)((D + 5) / 2) * 0x1p-23f;  // exact, >= 1 + (D + 4) 2^-24
    const bool far = __fmul_rd(lb, kLo) > __fadd_ru(__fmul_ru(ub_min, kHi), 0x1p-120f);
    return __ballot_sync(0xffffffffu, lane < k && !far);
}

// One cluster against the thread's PPT points: the reference's distance
// (t = x_f - c_f, fma(t, t, acc)) two points per packed op, and the strict
// '<' argmin update.
template <int D, int PPT>
__device__ __forceinline__ void dist_argmin(Tile<D, PPT>& T, float (&best)[PPT], const float2* __restrict__ cp,
                                            uint32_t c) {
    float2 cc[D];
#pragma unroll
    for (int f = 0; f < D; ++f) cc[f] = cp[f];
#pragma unroll
    for (int j = 0; j < PPT / 2; ++j) {
        float2 t = sub2(make_float2(T.x[0][2 * j], T.x[0][2 * j + 1]), cc[0]);
        float2 acc = mul2(t, t);  // == fma(t, t, 0) exactly
#pragma unroll
        for (int f = 1; f < D; ++f) {
            t = sub2(make_float2(T.x[f][2 * j], T.x[f][2 * j + 1]), cc[f]);
            acc = fma2(t, t, acc);
        }
        if (acc.x < best[2 * j]) {
            best[2 * j] = acc.x;
            T.lab[2 * j] = c;
        }
        if (acc.y < best[2 * j + 1]) {
            best[2 * j + 1] = acc.y;
            T.lab[2 * j + 1] = c;
        }
    }
}

template <int D, int PPT, int ACC, Pass PASS, int NT, bool PRUNE>
__device__ __forceinline__ void process_tile(Tile<D, PPT>& T, const FusedF32& a, uint64_t p0, bool vec,
                                             const float2* __restrict__ s_c, float* __restrict__ s_acc) {
    constexpr int VW = LowdCfg<D>::VW;
    const uint64_t n = a.n;
    const uint32_t k = a.k;

    if constexpr (PASS != Pass::SumsOnly) {
        float best[PPT];
#pragma unroll
        for (int i = 0; i < PPT; ++i) {
            best[i] = FLT_MAX;
            T.lab[i] = 0u;
        }
        if constexpr (PRUNE) {
            // the surviving clusters in ascending order: the same strict '<'
            // scan as below over a subset that holds every point's label
            uint32_t m = box_prune_mask<D, PPT>(T, p0, n, s_c, k);
            while (m) {
                const uint32_t c = __ffs(m) - 1;
                m &= m - 1;
                dist_argmin<D, PPT>(T, best, s_c + c * D, c);
            }
        } else {
            const float2* cp = s_c;
#pragma unroll 2
            for (uint32_t c = 0; c < k; ++c, cp += D) dist_argmin<D, PPT>(T, best, cp, c);
        }
        // labels out (unless the caller reads none this iteration)
        if (a.flags & FUSED_NO_LABELS) {
        } else if (vec && p0 + PPT <= n) {
#pragma unroll
            for (int v = 0; v < PPT; v += VW) {
                if constexpr (VW == 4) {
                    *reinterpret_cast<uint4*>(a.labels + p0 + v) =
                        make_uint4(T.lab[v], T.lab[v + 1], T.lab[v + 2], T.lab[v + 3]);
                } else if constexpr (VW == 2) {
                    *reinterpret_cast<uint2*>(a.labels + p0 + v) = make_uint2(T.lab[v], T.lab[v + 1]);
                } else {
                    a.labels[p0 + v] = T.lab[v];
                }
            }
        } else {
#pragma unroll
            for (int i = 0; i < PPT; ++i)
                if (p0 + i < n) a.labels[p0 + i] = T.lab[i];
        }
    }

    if constexpr (PASS != Pass::LabelOnly) {
        if constexpr (ACC == 3) {
            // private rows of VG-wide vectors: one vector load, packed adds and
            // one vector store per VG features, masses in their own column
            constexpr int VG = AccVec<D>::VG;
            constexpr int G = D / VG;
            float* srow0 = s_acc + (size_t)threadIdx.x * VG;
            unsigned int* mcol = reinterpret_cast<unsigned int*>(s_acc + (size_t)k * D * NT) + threadIdx.x;
#pragma unroll
            for (int i = 0; i < PPT; ++i) {
                const uint32_t l = T.lab[i];
                if (p0 + i < n && l < k) {
                    float* srow = srow0 + (size_t)l * G * NT * VG;
#pragma unroll
                    for (int g = 0; g < G; ++g) {
                        float* v = srow + (size_t)g * NT * VG;
                        if constexpr (VG == 4) {
                            float4 q = *reinterpret_cast<float4*>(v);
                            float2 lo = add2(make_float2(q.x, q.y), make_float2(T.x[4 * g][i], T.x[4 * g + 1][i]));
                            float2 hi = add2(make_float2(q.z, q.w), make_float2(T.x[4 * g + 2][i], T.x[4 * g + 3][i]));
                            *reinterpret_cast<float4*>(v) = make_float4(lo.x, lo.y, hi.x, hi.y);
                        } else if constexpr (VG == 2) {
                            float2 q = *reinterpret_cast<float2*>(v);
                            *reinterpret_cast<float2*>(v) = add2(q, make_float2(T.x[2 * g][i], T.x[2 * g + 1][i]));
                        } else {
                            *v += T.x[g][i];
                        }
                    }
                    mcol[(size_t)l * NT] += 1u;
                }
            }
        } else if constexpr (ACC == 0 || ACC == 2) {
            // private column per thread: no other thread touches it
            float* col = s_acc + threadIdx.x;
#pragma unroll
            for (int i = 0; i < PPT; ++i) {
                const uint32_t l = T.lab[i];
                if (p0 + i < n && l < k) {
                    float* row = col + (size_t)l * ((D + 1) * NT);
                    if constexpr (ACC == 0) {
#pragma unroll
                        for (int f = 0; f < D; ++f) row[f * NT] += T.x[f][i];
                        reinterpret_cast<unsigned int*>(row)[D * NT] += 1u;
                    } else {
#pragma unroll
                        for (int f = 0; f < D; ++f) atomicAdd(row + f * NT, T.x[f][i]);
                        atomicAdd(reinterpret_cast<unsigned int*>(row) + D * NT, 1u);
                    }
                }
            }
        } else {
            float* col = s_acc + (threadIdx.x & 31);
#pragma unroll
            for (int i = 0; i < PPT; ++i) {
                const uint32_t l = T.lab[i];
                if (p0 + i < n && l < k) {
                    float* row = col + (size_t)l * ((D + 1) * 32);
#pragma unroll
                    for (int f = 0; f < D; ++f) atomicAdd(row + f * 32, T.x[f][i]);
                    atomicAdd(reinterpret_cast<unsigned int*>(row) + D * 32, 1u);
                }
            }
        }
    }
}

template <int D, int PPT, int ACC, Pass PASS, int NT, int MINB, bool PREF, bool PRUNE = false>
__global__ void __launch_bounds__(NT, MINB)
    lowd_kernel(const FusedF32 a, const int vec_ok, const uint64_t ntiles) {
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t k = a.k;
    constexpr int W = (ACC == 1) ? 32 : NT;
    float2* s_c = reinterpret_cast<float2*>(smem);
    float* s_acc = reinterpret_cast<float*>(smem + (((size_t)k * D * sizeof(float2) + 15) & ~size_t(15)));

    if constexpr (PASS != Pass::SumsOnly) {
        for (uint32_t i = threadIdx.x; i < k * D; i += NT) {
            const uint32_t c = i / D, f = i - c * D;
            const float v = a.centroids[(size_t)f * k + c];
            s_c[i] = make_float2(v, v);
        }
    }
    if constexpr (PASS != Pass::LabelOnly) {
        const uint32_t words = k * (D + 1) * W;
        for (uint32_t i = threadIdx.x; i < words; i += NT) s_acc[i] = 0.0f;
    }
    __syncthreads();

    const bool vec = vec_ok != 0;
    constexpr uint64_t TILE = (uint64_t)NT * PPT;
    if constexpr (PREF) {
        // two tiles in flight per thread: the next tile's loads are issued
        // before the current tile is processed
        Tile<D, PPT> A, B;
        uint64_t t = blockIdx.x;
        if (t < ntiles) load_tile<D, PPT, PASS>(A, a, t * TILE + threadIdx.x * PPT, vec);
        while (t < ntiles) {
            const uint64_t t1 = t + gridDim.x;
            if (t1 < ntiles) load_tile<D, PPT, PASS>(B, a, t1 * TILE + threadIdx.x * PPT, vec);
            process_tile<D, PPT, ACC, PASS, NT, PRUNE>(A, a, t * TILE + threadIdx.x * PPT, vec, s_c, s_acc);
            if (t1 >= ntiles) break;
            const uint64_t t2 = t1 + gridDim.x;
            if (t2 < ntiles) load_tile<D, PPT, PASS>(A, a, t2 * TILE + threadIdx.x * PPT, vec);
            process_tile<D, PPT, ACC, PASS, NT, PRUNE>(B, a, t1 * TILE + threadIdx.x * PPT, vec, s_c, s_acc);
            t = t2;
        }
    } else {
        for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
            Tile<D, PPT> A;
            load_tile<D, PPT, PASS>(A, a, t * TILE + threadIdx.x * PPT, vec);
            process_tile<D, PPT, ACC, PASS, NT, PRUNE>(A, a, t * TILE + threadIdx.x * PPT, vec, s_c, s_acc);
        }
    }

    if constexpr (PASS == Pass::LabelOnly) {
        return;
    } else {
        __syncthreads();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const uint32_t entries = k * (D + 1);
        for (uint32_t e = warp; e < entries; e += NT / 32) {
            const uint32_t c = e / (D + 1), f = e - c * (D + 1);
            if constexpr (ACC == 3) {
                constexpr int VG = AccVec<D>::VG;
                constexpr int G = D / VG;
                if (f < D) {
                    const float* src = s_acc + ((size_t)(c * G + f / VG) * NT) * VG + (f % VG);
                    float v = 0.0f;
#pragma unroll 4
                    for (int j = lane; j < NT; j += 32) v += src[(size_t)j * VG];
                    v = warp_sum_f32(v);
                    if (lane == 0 && v != 0.0f) atomicAdd(&a.scratch.sums[(size_t)f * k + c], (double)v);
                } else {
                    const unsigned int* usrc = reinterpret_cast<const unsigned int*>(s_acc + (size_t)k * D * NT) + (size_t)c * NT;
                    unsigned int v = 0;
#pragma unroll 4
                    for (int j = lane; j < NT; j += 32) v += usrc[j];
                    v = __reduce_add_sync(0xffffffffu, v);
                    if (lane == 0 && v != 0u) atomicAdd(&a.scratch.masses[c], (unsigned long long)v);
                }
                continue;
            }
            const float* src = s_acc + (size_t)e * W;
            if (f < D) {
                float v = 0.0f;
#pragma unroll 4
                for (int j = lane; j < W; j += 32) v += src[j];
                v = warp_sum_f32(v);
                if (lane == 0 && v != 0.0f) atomicAdd(&a.scratch.sums[(size_t)f * k + c], (double)v);
            } else {
                unsigned int v = 0;
                const unsigned int* usrc = reinterpret_cast<const unsigned int*>(src);
#pragma unroll 4
                for (int j = lane; j < W; j += 32) v += usrc[j];
                v = __reduce_add_sync(0xffffffffu, v);
                if (lane == 0 && v != 0u) atomicAdd(&a.scratch.masses[c], (unsigned long long)v);
            }
        }
        if (a.mode == CKM_MODE_DEFER) return;
        if (last_cta_ticket(a.scratch.ctrl)) finalize_block<float, uint32_t>(D, k, a.new_centroids, a.masses, a.scratch, a.mode);
    }
}

size_t lowd_smem_bytes(uint32_t d, uint32_t k, int acc, Pass pass, int nt) {
    size_t b = (((size_t)k * d * sizeof(float2)) + 15) & ~size_t(15);
    if (pass != Pass::LabelOnly) b += (size_t)k * (d + 1) * (acc == 1 ? 32 : nt) * sizeof(float);
    return b;
}

constexpr size_t PRIVATE_TABLE_LIMIT = 100 * 1024;  // keeps two 256-thread CTAs per SM
constexpr size_t SHARED_TABLE_LIMIT = 200 * 1024;

int choose_acc(uint32_t d, uint32_t k, Pass pass) {
    if (pass == Pass::LabelOnly) return 0;
    if (lowd_smem_bytes(d, k, 0, pass, BLK) <= PRIVATE_TABLE_LIMIT) return 0;
    if (lowd_smem_bytes(d, k, 1, pass, BLK) <= SHARED_TABLE_LIMIT) return 1;
    return -1;
}

struct LaunchCache {
    std::mutex mu;
    std::unordered_map<const void*, int> attr_set;  // kernel -> max dynamic smem set
    std::unordered_map<uint64_t, int> occ;          // (kernel, smem) -> blocks per SM
};
LaunchCache& cache() {
    static LaunchCache c;
    return c;
}

template <int D, int PPT, int ACC, Pass PASS, int NT, int MINB, bool PREF, bool PRUNE = false>
int launch_lowd_v(const FusedF32& a, cudaStream_t s) {
    constexpr int VW = PPT < 4 ? PPT : 4;
    auto kern = lowd_kernel<D, PPT, ACC, PASS, NT, MINB, PREF, PRUNE>;
    const size_t smem = lowd_smem_bytes(D, a.k, ACC, PASS, NT);
    const DeviceInfo& di = device_info();
    if (smem > di.smem_optin) return fail(CKM_ERR_UNSUPPORTED, "lowd: shared-memory table too large");
    int blocks_per_sm = 0;
    {
        LaunchCache& C = cache();
        std::lock_guard<std::mutex> g(C.mu);
        const void* key = reinterpret_cast<const void*>(kern);
        auto it = C.attr_set.find(key);
        if (it == C.attr_set.end()) {
            // the dynamic limit is the opt-in maximum minus the static shared memory
            cudaFuncAttributes fa;
            cudaError_t e = cudaFuncGetAttributes(&fa, kern);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(lowd)");
            const int dyn_max = (int)(di.smem_optin - fa.sharedSizeBytes);
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(lowd)");
            it = C.attr_set.emplace(key, dyn_max).first;
        }
        if ((size_t)it->second < smem) return fail(CKM_ERR_UNSUPPORTED, "lowd: shared-memory table too large");
        const uint64_t okey = (reinterpret_cast<uint64_t>(key) << 20) ^ (uint64_t)smem;
        auto oi = C.occ.find(okey);
        if (oi == C.occ.end()) {
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, NT, smem);
            if (e != cudaSuccess) return cuda_fail(e, "occupancy(lowd)");
            if (blocks_per_sm < 1) return fail(CKM_ERR_UNSUPPORTED, "lowd: kernel does not fit on an SM");
            C.occ[okey] = blocks_per_sm;
        } else {
            blocks_per_sm = oi->second;
        }
    }
    const uint64_t tile = (uint64_t)NT * PPT;
    const uint64_t ntiles = (a.n + tile - 1) / tile;
    uint64_t grid = (uint64_t)di.sm_count * (uint64_t)blocks_per_sm;
    if (ntiles < grid) grid = ntiles;
    if (grid < 1) grid = 1;
    const uintptr_t pa = reinterpret_cast<uintptr_t>(a.points);
    const uintptr_t la = reinterpret_cast<uintptr_t>(a.labels);
    const int vec_ok = (a.n % VW == 0) && (pa % (VW * 4) == 0) && (la % (VW * 4) == 0);
    kern<<<(unsigned)grid, NT, smem, s>>>(a, vec_ok, ntiles);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "lowd launch");
    return CKM_OK;
}

// Tuning variants of the d = 4 fused pass, selected with the environment
// variable CKM_LOWD_VARIANT (default 0).  All variants compute the same
// result; they differ in points per thread, block size, prefetching and the
// accumulation table (0: private RMW, 1: lane columns shared by the CTA's
// warps with atomics, 2: private columns with atomic adds).  With box
// pruning: 11 no prefetch, 12 four points per thread, 13 128-thread CTAs.
int lowd_variant() {
    static int v = [] {
        const char* e = getenv("CKM_LOWD_VARIANT");
        return e ? atoi(e) : 0;
    }();
    return v;
}

int launch_d4_fused_variant(const FusedF32& a, cudaStream_t s, int v) {
    const size_t priv256 = lowd_smem_bytes(4, a.k, 0, Pass::Fused, 256);
    const size_t priv128 = lowd_smem_bytes(4, a.k, 0, Pass::Fused, 128);
    const size_t shared = lowd_smem_bytes(4, a.k, 1, Pass::Fused, 128);
    const bool prune = (a.flags & FUSED_BOX_PRUNE) && a.k <= 32;
    if (prune) {
        switch (v) {
            case 11: if (priv256 <= PRIVATE_TABLE_LIMIT) return launch_lowd_v<4, 8, 0, Pass::Fused, 256, 2, false, true>(a, s); break;
            case 12: if (priv256 <= PRIVATE_TABLE_LIMIT) return launch_lowd_v<4, 4, 0, Pass::Fused, 256, 2, true, true>(a, s); break;
            case 13: if (priv128 <= PRIVATE_TABLE_LIMIT / 2) return launch_lowd_v<4, 8, 0, Pass::Fused, 128, 4, false, true>(a, s); break;
            default: break;
        }
        return -1000;
    }
    switch (v) {
        case 7: if (priv128 <= PRIVATE_TABLE_LIMIT / 2) return launch_lowd_v<4, 8, 0, Pass::Fused, 128, 4, true>(a, s); break;
        case 9: if (priv256 <= PRIVATE_TABLE_LIMIT) return launch_lowd_v<4, 8, 0, Pass::Fused, 256, 2, true>(a, s); break;
        case 10: if (priv256 <= PRIVATE_TABLE_LIMIT) return launch_lowd_v<4, 8, 3, Pass::Fused, 256, 2, false>(a, s); break;
        default: break;
    }
    return -1000;  // not applicable: use the default
}

template <int D, Pass PASS>
int launch_lowd_acc(const FusedF32& a, cudaStream_t s) {
    constexpr int PPT = LowdCfg<D>::PPT;
    if constexpr (D == 4 && PASS == Pass::Fused) {
        const int v = lowd_variant();
        if (v != 0) {
            int st = launch_d4_fused_variant(a, s, v);
            if (st != -1000) return st;
        }
    }
    const int acc = choose_acc(D, a.k, PASS);
    if constexpr (PASS != Pass::SumsOnly && D <= 8) {
        if ((a.flags & FUSED_BOX_PRUNE) && a.k <= 32) {
            // pruned, the kernel waits on memory: the next tile's loads are
            // issued before the current tile is labelled (0.878 against
            // 0.944 ms per iteration at n = 2^28, d = 4, k = 16)
            if (acc == 0) return launch_lowd_v<D, PPT, 0, PASS, BLK, 2, true, true>(a, s);
            if (acc == 1) return launch_lowd_v<D, PPT, 1, PASS, BLK, 2, true, true>(a, s);
        }
    }
    if (acc == 0) return launch_lowd_v<D, PPT, 0, PASS, BLK, 2, false>(a, s);
    if (acc == 1) return launch_lowd_v<D, PPT, 1, PASS, BLK, 2, true>(a, s);
    return fail(CKM_ERR_UNSUPPORTED, "lowd: no accumulation layout fits");
}

template <Pass PASS>
int launch_lowd_pass(const FusedF32& a, cudaStream_t s) {
    switch (a.d) {
        case 1: return launch_lowd_acc<1, PASS>(a, s);
        case 2: return launch_lowd_acc<2, PASS>(a, s);
        case 3: return launch_lowd_acc<3, PASS>(a, s);
        case 4: return launch_lowd_acc<4, PASS>(a, s);
        case 5: return launch_lowd_acc<5, PASS>(a, s);
        case 6: return launch_lowd_acc<6, PASS>(a, s);
        case 7: return launch_lowd_acc<7, PASS>(a, s);
        case 8: return launch_lowd_acc<8, PASS>(a, s);
        case 12: return launch_lowd_acc<12, PASS>(a, s);
        case 16: return launch_lowd_acc<16, PASS>(a, s);
        default: return fail(CKM_ERR_UNSUPPORTED, "lowd: unsupported feature count");
    }
}

}  // namespace

bool lowd_supported(uint32_t d, uint32_t k) {
    if (k == 0) return false;
    if (!((d >= 1 && d <= 8) || d == 12 || d == 16)) return false;
    return choose_acc(d, k, Pass::Fused) >= 0;
}

int launch_fused_f32(const FusedF32& a, Pass pass, cudaStream_t s) {
    switch (pass) {
        case Pass::Fused: return launch_lowd_pass<Pass::Fused>(a, s);
        case Pass::LabelOnly: return launch_lowd_pass<Pass::LabelOnly>(a, s);
        case Pass::SumsOnly: return launch_lowd_pass<Pass::SumsOnly>(a, s);
    }
    return fail(CKM_ERR_INVALID_ARGUMENT, "bad pass");
}

}  // namespace ckm
