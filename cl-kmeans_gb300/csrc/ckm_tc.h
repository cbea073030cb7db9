// Tensor-core (tcgen05) Lloyd iteration: internal interface.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "ckm_internal.h"

namespace ckm {

struct TcLayout {
    uint32_t d_pad, k_pad;     // features padded to 64, clusters padded to 256
    uint64_t n_pad;            // points padded to 128
    size_t cent_rm_off, cent_bf16_off, cnorm2_off, cmax_off, flagged_off, counters_off, total;  // workspace
    size_t points_bf16_bytes, norms_bytes;                                       // prepared points
};
TcLayout tc_layout(uint64_t n, uint32_t d, uint32_t k);
bool tc_supported(uint32_t d, uint32_t k);

struct TcArgs {
    const float* points;        // FP32 column-major [d][n]
    const void* points_bf16;    // prepared: bf16 [n_pad][d_pad]
    const float* norms;         // prepared: [n_pad]
    const float* centroids;     // FP32 column-major [d][k]
    float* new_centroids;
    uint32_t* labels;
    uint32_t* masses;
    ScratchView scratch;
    void* workspace;            // tc_layout(n, d, k).total bytes
    unsigned int* stats;        // optional device [2]: rechecked points, error flag
    uint64_t n;
    uint32_t d, k;
    int mode;
};

int tc_prepare_points(const float* P, uint64_t n, uint32_t d, void* points_bf16, float* norms, cudaStream_t s);
int tc_iteration(const TcArgs& a, cudaStream_t s);

}  // namespace ckm
