// Device-side descriptors of the batched Lloyd kernel.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

struct ckm_batch;  // include/ckm.h

namespace ckm {

// Jobs of d = 32 or 64 with UMMA_MIN_K <= k <= UMMA_MAX_K may take the batched
// kernel's tensor-core path (N of one tcgen05.mma is at most 256; below 16
// clusters the FP32 screen is faster).
constexpr uint32_t UMMA_MIN_K = 16;
constexpr uint32_t UMMA_MAX_K = 256;

// Per-job state kept on the device between iterations.
struct BatchStatus {
    float shift;          // max |new - old| / max |old| of the last iteration
    uint32_t iterations;  // iterations finished
    uint32_t parity;      // centroids live in cent[parity]; flipped by the finalising CTA
    uint32_t flags;       // bit 0: inactive (skipped by the step); bit 1: finished (converged or max iterations);
                          // bit 2: failed (a bounded wait for the tensor cores ran out)
};

struct BatchJobDev {
    const float* points;        // column-major n x d
    float* cent[2];             // centroid double buffer, column-major k x d
    uint32_t* labels;
    uint32_t* masses;
    double* sums;               // FP64 scratch [f * k + c]
    unsigned long long* msum;   // [k]
    unsigned int* ticket;       // tiles merged this iteration
    BatchStatus* status;
    uint64_t n;
    uint32_t d, k;
    uint32_t num_tiles;
    uint32_t pad;
};

// A contiguous run of one job's tiles: one unit of work, claimed by a CTA.
struct BatchSegment {
    uint32_t job, tile_begin, tile_end, pad;
};

// One step: the CTAs claim segments in list order (largest first) from the
// counter *work, which the launch resets to zero beforehand.  tol > 0 /
// max_it > 0: a job whose shift falls below tol, or that has run max_it
// iterations, parks itself (status flags bits 0 and 1).
// block: threads per CTA, 256 or 512.  use_umma bit 0 (512-thread CTAs, one
// per SM): d = 32 / 64 segments may take the tensor-core path, each CTA
// holding 512 TMEM columns; bit 1: failure-detection test (the tensor-core
// waits run out after 1 ms and the jobs are parked as failed).
int launch_batched(const BatchJobDev* jobs, const BatchSegment* segs, uint32_t num_segs, unsigned int* work,
                   float tol, uint32_t max_it, uint32_t grid, uint32_t block, uint32_t tile, uint32_t flush_tiles,
                   size_t cent_cap, size_t acc_cap, uint32_t use_umma, cudaStream_t s);
int batched_blocks_per_sm(size_t smem, uint32_t block, int* out);
// Copies cent[1] into cent[0] for every job whose parity is 1 and resets the
// parity, so the caller's centroid arrays hold the current centroids.
int launch_batch_sync(const BatchJobDev* jobs, uint32_t num_jobs, cudaStream_t s);

// Batches over job state owned by the caller (the serving loop keeps each
// job's buffers, scratch and status for its whole life): the job table is
// replaced and the schedule rebuilt each round; the batch allocates only its
// table, work list and counter.
int batch_create_external(::ckm_batch** out);
int batch_set_jobs(::ckm_batch* b, const BatchJobDev* jobs, uint32_t num_jobs, uint32_t tile, uint32_t ctas_per_sm,
                   float tol, uint32_t max_it, cudaStream_t s);
int batch_launch_step(::ckm_batch* b, cudaStream_t s);

}  // namespace ckm
