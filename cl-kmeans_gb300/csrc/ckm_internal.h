// Internal declarations shared by the CUDA translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

#include "../../include/ckm.h"

namespace ckm {

// Last-error message of the calling host thread.
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t err, const char* where);

// Scratch layout (all offsets 256-byte aligned):
//   sums     double[k * d]   column-major like the centroids (f * k + c)
//   masses   uint64[k]
//   control  uint32[64]      [0] CTA arrival ticket, [1] error flag
//   ext      FUSED_UMMA_EXT bytes, only for the shapes the fused call may run
//            on the tensor cores (d = 32 / 64, 16 <= k <= 256): the one-job
//            record, status, tile ticket, work counter and segment list of
//            the batched kernel (ckm_batched.cu, launch_fused_umma)
constexpr size_t FUSED_UMMA_EXT = 4096;
struct ScratchLayout {
    size_t sums_off, mass_off, ctrl_off, ext_off, total;  // ext_off 0: no extension
};
ScratchLayout scratch_layout(uint32_t d, uint32_t k);

struct ScratchView {
    double* sums;
    unsigned long long* masses;
    unsigned int* ctrl;
    unsigned char* ext;  // nullptr without the extension
};
inline ScratchView scratch_view(void* base, const ScratchLayout& L) {
    char* b = static_cast<char*>(base);
    return ScratchView{reinterpret_cast<double*>(b + L.sums_off),
                       reinterpret_cast<unsigned long long*>(b + L.mass_off),
                       reinterpret_cast<unsigned int*>(b + L.ctrl_off),
                       L.ext_off ? reinterpret_cast<unsigned char*>(b + L.ext_off) : nullptr};
}

// Counts kernel launches made by this library (for the run info and bench).
void count_launch(uint64_t n = 1);
uint64_t launch_count();

// Device properties cached per device.
struct DeviceInfo {
    int sm_count;
    size_t smem_optin;          // per block (opt-in maximum)
    size_t smem_per_sm;         // per multiprocessor
    size_t smem_reserved;       // reserved by the system per block
    int cc_major, cc_minor;
};
const DeviceInfo& device_info();

// Work of one fused / labeling / centroid-update launch (f32).
struct FusedF32 {
    const float* points;
    const float* centroids;       // old centroids (column-major)
    uint32_t* labels;             // written by fused / labeling; read by centroid update
    float* new_centroids;         // FINALIZE: means, ACCUMULATE: += sums
    uint32_t* masses;             // FINALIZE: counts, ACCUMULATE: += counts
    ScratchView scratch;
    uint64_t n;
    uint32_t d, k;
    int mode;
    // FUSED_BOX_PRUNE: per warp, skip the clusters that are provably farther
    // than another one from every point of the warp (points in spatial order,
    // e.g. from spatial_sort, make this effective); labels are unchanged.
    uint32_t flags = 0;
};

constexpr uint32_t FUSED_BOX_PRUNE = 1u;
// FUSED_NO_LABELS: the low-d fused pass writes no labels (a caller whose
// labels of this iteration nobody reads; the sums and masses are the same).
constexpr uint32_t FUSED_NO_LABELS = 2u;

struct FusedF64 {
    const double* points;
    const double* centroids;
    uint64_t* labels;
    double* new_centroids;
    uint64_t* masses;
    ScratchView scratch;
    uint64_t n;
    uint32_t d, k;
    int mode;
};

enum class Pass { Fused, LabelOnly, SumsOnly };

// Launchers (return CKM_OK or an error status; never throw).
int launch_fused_f32(const FusedF32& a, Pass pass, cudaStream_t s);
// The fused iteration (FINALIZE) of one d = 32 / 64 job on the batched
// kernel's tensor-core path; -1000 when the shape, device or scratch does
// not qualify (the caller takes another kernel).
int launch_fused_umma(const FusedF32& a, cudaStream_t s);
// Spatial order (ckm_spatial.cu): radix sort by a Z-order cell key.
size_t spatial_sort_workspace_bytes(uint64_t n, uint32_t d);
int launch_spatial_sort(uint32_t d, uint64_t n, const float* points, float* sorted, uint32_t* perm, void* ws,
                        cudaStream_t s);
int launch_unpermute_u32(uint64_t n, const uint32_t* perm, const uint32_t* in, uint32_t* out, cudaStream_t s);
int launch_generic_f32(const FusedF32& a, Pass pass, cudaStream_t s);
int launch_generic_f64(const FusedF64& a, Pass pass, cudaStream_t s);
bool lowd_supported(uint32_t d, uint32_t k);

int launch_finalize_f32(uint32_t d, uint32_t k, float* c, uint32_t* m, ScratchView sv, int mode,
                        cudaStream_t s);
int launch_finalize_f64(uint32_t d, uint32_t k, double* c, uint64_t* m, ScratchView sv, int mode,
                        cudaStream_t s);
int launch_mass_u32(uint64_t n, uint32_t k, const uint32_t* labels, uint32_t* masses, cudaStream_t s);
int launch_mass_u64(uint64_t n, uint32_t k, const uint64_t* labels, uint64_t* masses, cudaStream_t s);
int launch_shift_f32(uint64_t kd, const float* o, const float* n, float* out, cudaStream_t s);
int launch_shift_f64(uint64_t kd, const double* o, const double* n, float* out, cudaStream_t s);
int launch_divide_f32(uint32_t d, uint32_t k, float* m, const uint32_t* masses, cudaStream_t s);
int launch_divide_f64(uint32_t d, uint32_t k, double* m, const uint64_t* masses, cudaStream_t s);
template <typename T>
int launch_add(uint64_t count, T* a, const T* b, cudaStream_t s);
int launch_reduce_parcol_u32(uint64_t cols, uint64_t rows, uint32_t* data, cudaStream_t s);
int launch_generate_f32(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed, float clo, float chi,
                        float slo, float shi, uint64_t first, float* out, uint64_t stride,
                        cudaStream_t s);
int launch_generate_ex_f32(uint32_t d, uint64_t n, uint32_t blobs, uint64_t seed, int center_dist, float ca,
                           float cb, int sigma_dist, float slo, float shi, int dirichlet, uint64_t first, float* out,
                           uint64_t stride, cudaStream_t s);

}  // namespace ckm
