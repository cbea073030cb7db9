// Tensor-core (tcgen05) Lloyd iteration: internal interface.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "ckm_internal.h"

namespace ckm {

// Header at the start of a prepared point set (device memory, 256 bytes).
struct TcPointsHeader {
    unsigned int maxabs_bits;  // max |x_f| over the finite coordinates (float bits)
    uint32_t precision;        // operand type of the distance GEMM: CKM_TC_FP16 or CKM_TC_BF16
    uint32_t reserved[62];
};

// Per-iteration device values (start of the workspace, 256 bytes).
struct TcIterDev {
    unsigned int nflagged;     // points sent to the full exact recheck
    unsigned int error;        // nonzero: a bounded device wait ran out
    unsigned int resolved;     // points with 2+ candidates (resolved exactly after labeling)
    unsigned int overflowed;   // points whose candidate list overflowed (part of nflagged)
    unsigned int cabs_bits;    // max |c_f| over valid centroids (float bits)
    unsigned int cmax_bits;    // upper bound of max |c| over valid centroids (float bits)
    unsigned int fmax_bits;    // upper bound of max |fp16(c) / sc - c| over valid centroids (float bits)
    float alpha;               // score = cn2 + alpha * (fp16 dot product)
    float t0, t1, te, t2, cm;  // threshold T = t0 + t1 |x| + te |e| + t2 (|x| + cm)^2, e = fp16 error of x
    uint32_t reserved[50];
};

struct TcLayout {
    uint32_t d_pad;            // features padded to 64 (one 128-byte swizzle row of fp16)
    uint32_t d4;               // features padded to 4 (FP32 row-major copies)
    uint32_t k_pad;            // clusters padded to a whole chunk
    uint32_t bn;               // clusters per chunk (TMEM columns per accumulator)
    uint64_t n_pad;            // points padded to a pair of 128-point tiles
    // prepared points (ckm_tc_points_bytes), all in the set's own point order:
    // fp16 rows, bounds of |x| and of its fp16 rounding error, FP32 rows, and
    // the caller's index of each point
    size_t pts_half_off, pts_norm_off, pts_err_off, pts_rm_off, pts_orig_off, pts_total;
    // per-iteration workspace (ckm_tc_workspace_bytes)
    size_t ws_cent_rm_off, ws_cent_half_off, ws_cn2_off, ws_flagged_off, ws_off_off, ws_cursor_off, ws_perm_off,
        ws_slabels_off, ws_res_pts_off, ws_res_cands_off, ws_total;
};
TcLayout tc_layout(uint64_t n, uint32_t d, uint32_t k);
bool tc_supported(uint32_t d, uint32_t k);

struct TcArgs {
    const float* points;        // FP32 column-major [d][n]
    const void* tc_points;      // prepared point set (tc_prepare_points)
    const float* centroids;     // FP32 column-major [d][k]
    float* new_centroids;
    uint32_t* labels;
    uint32_t* masses;
    ScratchView scratch;
    void* workspace;            // tc_layout(n, d, k).ws_total bytes
    unsigned int* stats;        // optional device [2]: rechecked points, error flag
    uint64_t n;
    uint32_t d, k;
    int mode;
};

int tc_prepare_points(const float* P, uint64_t n, uint32_t d, void* tc_points, int precision, cudaStream_t s);
// dst = src reordered by the label order of the last iteration run with `workspace`
int tc_sort_points(uint64_t n, uint32_t d, uint32_t k, const void* src, void* dst, const void* workspace,
                   cudaStream_t s);
int tc_iteration(const TcArgs& a, cudaStream_t s);

}  // namespace ckm
