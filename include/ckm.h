/*
 * ckm.h -- C ABI of the GB300 Lloyd k-means library (libckm.so).
 *
 * Drop-in boundary for the reference's Lloyd iteration path.  The reference
 * binds its kernels through C++ std::function factories over Boost.Compute
 * buffers; each entry point below replaces one of those functors (the
 * replaced interface is cited at each declaration).  Everything is plain
 * pointers, sizes and a CUDA stream; nothing allocates on the hot calls.
 *
 * Layouts follow the reference (lloyd_fused_feature_sum.cl:77-79, 200, 230):
 *   points     column-major  P[f * num_points + p]      (PointT)
 *   centroids  column-major  C[f * num_clusters + c]    (PointT)
 *   labels     LabelT[num_points]
 *   masses     MassT[num_clusters]
 * Type pairs: float/uint32/uint32 (_f32) and double/uint64/uint64 (_f64),
 * the two instantiations bench.cpp:469-503 dispatches.
 *
 * Semantics kept from the reference:
 *   - distance = fma(x_f - c_f, x_f - c_f, acc) over f = 0..d-1 from 0,
 *     argmin with strict '<' from cluster 0 with min = type max and label 0:
 *     the lowest index wins a tie and a NaN distance never wins
 *     (kmeans_naive.cpp:48-63, lloyd_fused_feature_sum.cl:209-239);
 *   - an empty cluster divides 0 by 0 and gets NaN centroids
 *     (kmeans_naive.cpp:96-100, matrix_binary_op.cl:98-114);
 *   - functor-level calls ACCUMULATE into new_centroids / masses, the caller
 *     zero-fills (kmeans_single_stage.hpp:97-112, fused_feature_sum.hpp:403-439).
 *
 * Every function returns a status: CKM_OK (0) or a negative ckm_status.  No
 * exception crosses this boundary; ckm_last_error() has the message.
 */
#ifndef CKM_H
#define CKM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ABI-identical to cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st *ckm_stream_t;

typedef enum ckm_status {
    CKM_OK = 0,
    CKM_ERR_INVALID_ARGUMENT = -1,  /* the reference's size asserts, fused_feature_sum.hpp:210-220 */
    CKM_ERR_UNSUPPORTED = -2,
    CKM_ERR_SCRATCH_TOO_SMALL = -3,
    CKM_ERR_CUDA = -4,
    CKM_ERR_ALLOC = -5,
    CKM_ERR_IO = -6,
    CKM_ERR_TIMEOUT = -7,           /* a bounded device wait ran out */
    CKM_ERR_UNKNOWN_STRATEGY = -8,  /* the factories' std::invalid_argument(strategy) */
    CKM_ERR_CANCELLED = -9,
    CKM_ERR_BUDGET = -10            /* device-memory budget would be exceeded */
} ckm_status;

/* Fused-call modes.  CKM_MODE_ACCUMULATE is the reference FusedFunction
 * contract (+= into new_centroids sums and masses).  CKM_MODE_FINALIZE runs a
 * whole Lloyd iteration in one launch: new_centroids = means, masses = counts
 * (what fill -> fused -> reduce -> add -> matrix_divide.row computes,
 * kmeans_single_stage.hpp:97-144).  CKM_MODE_DEFER only accumulates into the
 * FP64 scratch; ckm_finalize_* turns it into centroids later (chunked runs). */
enum {
    CKM_MODE_DEFER = 0,
    CKM_MODE_FINALIZE = 1,
    CKM_MODE_ACCUMULATE = 2
};

const char *ckm_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char *ckm_last_error(void);
/* Library ABI version (major * 10000 + minor * 100 + patch). */
int ckm_version(void);
/* Number of CUDA devices the library sees (CKM_ERR_CUDA when none). */
int ckm_device_count(int *count);
/* Kernels this library has launched in this process (all threads). */
uint64_t ckm_launch_count(void);
/* The C++ strategies (ckm_kmeans_run_f32 / _f64 and the bench) take their
 * device buffers from the current device's default stream-ordered pool and
 * keep freed memory there for the next run.  This waits for the device and
 * returns that cached memory to the system. */
int ckm_release_cached_memory(void);

/* ---------------------------------------------------------------------- */
/* Scratch.  The fused, centroid-update and finalize calls merge per-CTA   */
/* partial sums in FP64 into caller-owned scratch (this replaces the        */
/* reference's global partial buffers + ReduceVectorParcol,                */
/* fused_feature_sum.hpp:224-307, 391-425).  Size it with                   */
/* ckm_scratch_bytes, zero it once with ckm_scratch_init; every call that   */
/* finalizes or accumulates leaves it zeroed again.  Calls that share one   */
/* scratch must be stream-ordered.                                          */
/* ---------------------------------------------------------------------- */
size_t ckm_scratch_bytes(uint32_t num_features, uint32_t num_clusters);
int ckm_scratch_init(void *scratch, size_t scratch_bytes, ckm_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Fused single pass: label + mass + feature sums (+ merge, + divide).      */
/* Replaces FusedFactory::FusedFunction (fused_factory.hpp:34-53), i.e.     */
/* FusedFeatureSum::operator() (cl_kernels/fused_feature_sum.hpp:191-444)   */
/* and FusedClusterMerge::operator() (cl_kernels/fused_cluster_merge.hpp:   */
/* 193-414).  ckm_fused_f32 picks its kernel by shape: d <= 16 the low-d    */
/* kernel; d = 32 / 64 the rows kernel, or, in FINALIZE mode with k >= 128  */
/* and n >= 2^20, one job of the batched kernel's tcgen05 path (its records */
/* in a 4 KiB part of the scratch that ckm_scratch_bytes includes for       */
/* d = 32 / 64 with 16 <= k <= 256); otherwise the generic kernel.  The     */
/* labels are the reference's on every path.                                */
/* ---------------------------------------------------------------------- */
int ckm_fused_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                  const float *points, const float *old_centroids, float *new_centroids,
                  uint32_t *labels, uint32_t *masses, void *scratch, size_t scratch_bytes,
                  int mode, ckm_stream_t stream);
int ckm_fused_f64(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                  const double *points, const double *old_centroids, double *new_centroids,
                  uint64_t *labels, uint64_t *masses, void *scratch, size_t scratch_bytes,
                  int mode, ckm_stream_t stream);

/* Spatially ordered point sets (no counterpart in the reference; a layout
 * of the same points).  ckm_spatial_sort_f32 writes a copy of the
 * column-major points in Z-order of 2^16 cells of their bounding box, taken
 * over a strided sample of 2^20 points (points outside it fall in the edge
 * cells) (1 <= d <= 16, n < 2^32; a stable radix sort, so equal cells keep
 * the caller's order) and, when perm is not NULL, perm[q] = the caller's
 * index of sorted point q.  Its workspace holds one more copy of the points,
 * two 16-bit keys per point and the indices:
 * ckm_spatial_sort_workspace_bytes(n, d) bytes.
 * ckm_fused_sorted_f32 is ckm_fused_f32 (same contract, same labels, masses
 * and centroids for the points it is given) that, for d <= 8 and k <= 32,
 * skips per warp the clusters provably farther than another from all of the
 * warp's points; on a spatially ordered set most clusters are skipped.  Its
 * labels follow the order of the points it is given; ckm_unpermute_u32
 * brings them to the caller's order (out[perm[q]] = in[q]).  For d <= 16,
 * labels may be NULL: none are written (an iteration whose labels nobody
 * reads, e.g. every iteration but the last of a fixed-length run); masses
 * and centroids are unchanged. */
size_t ckm_spatial_sort_workspace_bytes(uint64_t num_points, uint32_t num_features);
int ckm_spatial_sort_f32(uint32_t num_features, uint64_t num_points, const float *points, float *sorted_points,
                         uint32_t *perm, void *workspace, size_t workspace_bytes, ckm_stream_t stream);
int ckm_fused_sorted_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                         const float *points, const float *old_centroids, float *new_centroids,
                         uint32_t *labels, uint32_t *masses, void *scratch, size_t scratch_bytes,
                         int mode, ckm_stream_t stream);
/* ckm_labeling_f32 with the same per-warp box pruning (labels unchanged). */
int ckm_labeling_sorted_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                            const float *points, const float *centroids, uint32_t *labels, ckm_stream_t stream);
int ckm_unpermute_u32(uint64_t num_points, const uint32_t *perm, const uint32_t *in, uint32_t *out,
                      ckm_stream_t stream);

/* The same fused iteration for callers that cannot allocate device memory
 * (a plugin inside a framework that owns all device memory, a loop that
 * must never call cudaMalloc/cudaFree, a caller given only its buffers).
 * No counterpart in the reference: its functors allocate their own partial
 * buffers.  The FP64 merge scratch is a built-in 128 KiB device array
 * instead of an argument, which caps ckm_scratch_bytes(d, k) at 128 KiB
 * (about k*d <= 15,000; larger sizes return CKM_ERR_SCRATCH_TOO_SMALL).
 * mode: CKM_MODE_FINALIZE or CKM_MODE_ACCUMULATE.  The array is shared by
 * all calls on a device: calls that may overlap on the GPU race, so keep
 * them on one stream.  Each call clears the part it uses first.  The first
 * call in each CUDA context (on each device, and again after cudaDeviceReset
 * or a switch to another context) looks up the array's address
 * (cudaGetSymbolAddress); make it before any stream capture. */
int ckm_fused_f32_noalloc(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                          const float *points, const float *old_centroids, float *new_centroids,
                          uint32_t *labels, uint32_t *masses, int mode, ckm_stream_t stream);

/* Tensor-core fused iteration for large k*d (d <= 256): the same contract as
 * ckm_fused_f32, computed as an fp16 distance GEMM on the tensor cores
 * (tcgen05, f32 accumulation; operands scaled by powers of two), whose labels
 * are certified against a rigorous error bound; the clusters the bound cannot
 * separate are recomputed with the reference's exact FP32 arithmetic, so the
 * labels are the reference's.  Sums merge in FP64.  Replaces the same functor as
 * ckm_fused_f32 (fused_factory.hpp:34-53) for shapes where the distance
 * block is a dense contraction.
 *   tc_points: ckm_tc_points_bytes(n, d) bytes, filled once per point set by
 *              ckm_tc_prepare_points (scaled fp16 rows, FP32 rows, norm
 *              bounds, point indices), or by ckm_tc_sort_points;
 *   workspace: ckm_tc_workspace_bytes(n, d, k) bytes;
 *   stats:     optional device uint32[2]: points rechecked exactly, and a
 *              nonzero error flag if a bounded device wait ran out. */
size_t ckm_tc_points_bytes(uint64_t num_points, uint32_t num_features);
size_t ckm_tc_workspace_bytes(uint64_t num_points, uint32_t num_features, uint32_t num_clusters);
int ckm_tc_supported(uint32_t num_features, uint32_t num_clusters);
int ckm_tc_prepare_points(uint32_t num_features, uint64_t num_points, const float *points, void *tc_points,
                          size_t tc_points_bytes, ckm_stream_t stream);
/* The same with the operand type of the distance GEMM chosen: CKM_TC_FP16
 * (the default: fp16 operands scaled by powers of two) or CKM_TC_BF16.  The
 * certificate is built from the operands' measured rounding errors, so both
 * give the reference's labels; bf16's coarser rounding leaves more points to
 * the exact resolution (a slower iteration on typical data).  Same functor
 * as ckm_tc_prepare_points (fused_factory.hpp:34-53). */
#define CKM_TC_FP16 0
#define CKM_TC_BF16 1
int ckm_tc_prepare_points_ex(uint32_t num_features, uint64_t num_points, const float *points, void *tc_points,
                             size_t tc_points_bytes, int precision, ckm_stream_t stream);
/* Diagnostics of the last ckm_tc_fused_f32 call made with `workspace`:
 * copies to the device array counters[4] (stream-ordered) the number of
 * points sent to the full exact recheck, the error flag, the number of
 * points resolved among 2+ candidates in the label kernel, and the number of
 * points whose candidate list overflowed (counted in the first value too). */
int ckm_tc_counters(const void *workspace, uint32_t *counters, ckm_stream_t stream);

/* Writes into sorted_tc_points (its own ckm_tc_points_bytes(n, d) buffer) the
 * prepared set tc_points reordered by the clusters of the last
 * ckm_tc_fused_f32 call made with `workspace` for the same set and k.  Points
 * of one cluster then share the label kernel's 128-point tiles, which keeps
 * its candidate tests coherent across a warp.  Labels, masses and centroids
 * stay in the caller's point order: the set carries each point's index.  No
 * counterpart in the reference. */
int ckm_tc_sort_points(uint32_t num_features, uint64_t num_points, uint32_t num_clusters, const void *tc_points,
                       void *sorted_tc_points, size_t tc_points_bytes, const void *workspace,
                       size_t workspace_bytes, ckm_stream_t stream);
int ckm_tc_fused_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters, const float *points,
                     const void *tc_points, const float *old_centroids, float *new_centroids, uint32_t *labels,
                     uint32_t *masses, void *scratch, size_t scratch_bytes, void *workspace,
                     size_t workspace_bytes, int mode, uint32_t *stats, ckm_stream_t stream);

/* Labels only.  Replaces LabelingFactory::LabelingFunction
 * (labeling_factory.hpp:33-48) = LabelingUnrollVector::operator()
 * (cl_kernels/labeling_unroll_vector.hpp:168-272). */
int ckm_labeling_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                     const float *points, const float *centroids, uint32_t *labels,
                     ckm_stream_t stream);
int ckm_labeling_f64(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                     const double *points, const double *centroids, uint64_t *labels,
                     ckm_stream_t stream);

/* Label histogram, += into masses.  Replaces
 * MassUpdateFactory::MassUpdateFunction (mass_update_factory.hpp:36-48) for
 * all four strategies (cl_kernels/mass_update_{global_atomic,part_global,
 * part_local,part_private}.hpp).  Exact integer counts. */
int ckm_mass_update_u32(uint64_t num_points, uint32_t num_clusters, const uint32_t *labels,
                        uint32_t *masses, ckm_stream_t stream);
int ckm_mass_update_u64(uint64_t num_points, uint32_t num_clusters, const uint64_t *labels,
                        uint64_t *masses, ckm_stream_t stream);

/* Per-label feature sums, += into centroids (the caller zero-fills and then
 * divides).  Replaces CentroidUpdateFactory::CentroidUpdateFunction
 * (centroid_update_factory.hpp:37-54) for feature_sum, feature_sum_pardim
 * and cluster_merge (cl_kernels/centroid_update_*.hpp).  `masses` is the
 * reference argument and is not modified.  mode CKM_MODE_DEFER keeps the
 * sums in scratch (for chunked runs), CKM_MODE_ACCUMULATE adds them into
 * centroids (reference contract). */
int ckm_centroid_update_f32(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                            const float *points, float *centroids, const uint32_t *labels,
                            const uint32_t *masses, void *scratch, size_t scratch_bytes,
                            int mode, ckm_stream_t stream);
int ckm_centroid_update_f64(uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                            const double *points, double *centroids, const uint64_t *labels,
                            const uint64_t *masses, void *scratch, size_t scratch_bytes,
                            int mode, ckm_stream_t stream);

/* Relative centroid shift of one iteration, written to the device float
 * *shift: max |new - old| over max |old| (NaN entries, empty clusters, are
 * skipped).  The convergence test of `kmeans.converge` (parsed but unused
 * in the reference, configuration_parser.cpp:67, 143-145). */
int ckm_centroid_shift_f32(uint32_t num_features, uint32_t num_clusters, const float *old_centroids,
                           const float *new_centroids, float *shift, ckm_stream_t stream);
int ckm_centroid_shift_f64(uint32_t num_features, uint32_t num_clusters, const double *old_centroids,
                           const double *new_centroids, float *shift, ckm_stream_t stream);

/* M[f*k + c] = M[f*k + c] / (PointT) masses[c].  Replaces
 * MatrixBinaryOp<PointT,MassT>::row with Divide
 * (cl_kernels/matrix_binary_op.hpp:86-127; matrix_binary_op.cl:98-114). */
int ckm_matrix_divide_row_f32(uint32_t num_features, uint32_t num_clusters, float *matrix,
                              const uint32_t *masses, ckm_stream_t stream);
int ckm_matrix_divide_row_f64(uint32_t num_features, uint32_t num_clusters, double *matrix,
                              const uint64_t *masses, ckm_stream_t stream);

/* A[i] += B[i].  Replaces MatrixBinaryOp::matrix with Add
 * (cl_kernels/matrix_binary_op.hpp:149-188; matrix_binary_op.cl:126-140). */
int ckm_matrix_add_f32(uint64_t count, float *a, const float *b, ckm_stream_t stream);
int ckm_matrix_add_f64(uint64_t count, double *a, const double *b, ckm_stream_t stream);
int ckm_matrix_add_u32(uint64_t count, uint32_t *a, const uint32_t *b, ckm_stream_t stream);
int ckm_matrix_add_u64(uint64_t count, uint64_t *a, const uint64_t *b, ckm_stream_t stream);

/* Column sums of `num_cols` vectors of `num_rows` uint32 (column-major),
 * wrapping mod 2^32, into the first num_rows entries of `data`.  Replaces
 * ReduceVectorParcol (cl_kernels/reduce_vector_parcol.hpp:64-155), which the
 * reference's test/reduce_vector.cpp pins. */
int ckm_reduce_vector_parcol_u32(uint64_t num_cols, uint64_t num_rows, uint32_t *data,
                                 ckm_stream_t stream);

/* Turns the FP64 sums of CKM_MODE_DEFER calls into centroids and masses
 * (centroids = sums / masses; 0/0 -> NaN) and re-zeroes the scratch.  The
 * matrix_divide.row step of the buffered strategies
 * (kmeans_single_stage_buffered.hpp:230-244). */
int ckm_finalize_f32(uint32_t num_features, uint32_t num_clusters, float *new_centroids,
                     uint32_t *masses, void *scratch, size_t scratch_bytes, ckm_stream_t stream);
int ckm_finalize_f64(uint32_t num_features, uint32_t num_clusters, double *new_centroids,
                     uint64_t *masses, void *scratch, size_t scratch_bytes, ckm_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Seeded synthetic Gaussian mixture (counter-based Philox4x32-10), column- */
/* major, generated on the device.  Stands in for the reference's           */
/* cluster_generator.cpp:157-196 file writer.  Blob centres are uniform in  */
/* [center_lo, center_hi]^d, blob sigmas uniform in [sigma_lo, sigma_hi],   */
/* components equally likely; point p depends only on (seed, p).            */
/* ---------------------------------------------------------------------- */
int ckm_generate_mixture_f32(uint32_t num_features, uint64_t num_points, uint32_t num_blobs,
                             uint64_t seed, float center_lo, float center_hi, float sigma_lo,
                             float sigma_hi, uint64_t first_point, float *points,
                             uint64_t points_stride, ckm_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Batched jobs: many independent k-means problems of uneven size advanced  */
/* by ONE persistent kernel launch per iteration.  No counterpart in the    */
/* reference (it runs one problem per bench invocation).  The handle owns   */
/* the device job table, the CTA schedule and every job's FP64 scratch and  */
/* second centroid buffer, all allocated by ckm_batch_create; stepping      */
/* allocates nothing.  Each job's arrays are the caller's device arrays.    */
/* ---------------------------------------------------------------------- */
typedef struct ckm_batch_job {
    const float *points;    /* device, column-major num_points x num_features */
    float *centroids;       /* device, column-major num_clusters x num_features; in: initial */
    uint32_t *labels;       /* device [num_points], out */
    uint32_t *masses;       /* device [num_clusters], out */
    uint64_t num_points;
    uint32_t num_features;
    uint32_t num_clusters;
} ckm_batch_job;

typedef struct ckm_batch_options {
    uint32_t tile_points;   /* points per tile; 0 = choose (autotune or default) */
    uint32_t ctas_per_sm;   /* 0 = choose; 1 = one 512-thread CTA per SM (d = 32 / 64 jobs with
                               16 <= k <= 256 then label on the tcgen05 tensor cores), 2 or more =
                               256-thread CTAs (TF32 mma.sync screen for d = 32 / 64) */
    uint32_t flush_tiles;   /* tiles between FP64 merges of a CTA's partial sums; 0 = 16 */
    int autotune;           /* time candidate tile sizes / CTA counts on the batch itself */
    float tolerance;        /* > 0: a job stops (is skipped by later steps) once its relative centroid
                               shift falls below this (the kmeans.converge test) */
    uint32_t max_iterations;/* > 0: a job stops after this many iterations */
} ckm_batch_options;

typedef struct ckm_batch ckm_batch;

/* Uploads the job table and builds a cost-balanced schedule.  jobs may be
 * freed after the call; the device arrays they point to must stay alive. */
int ckm_batch_create(const ckm_batch_job *jobs, uint32_t num_jobs, const ckm_batch_options *options,
                     ckm_batch **out, ckm_stream_t stream);
/* One Lloyd iteration of every active job: one kernel launch. */
int ckm_batch_step(ckm_batch *batch, ckm_stream_t stream);
/* `iterations` steps (captured once into a CUDA graph and replayed when
 * use_graph != 0), then brings every job's current centroids into its
 * `centroids` array. */
int ckm_batch_run(ckm_batch *batch, uint32_t iterations, int use_graph, ckm_stream_t stream);
/* Brings the current centroids into the jobs' `centroids` arrays. */
int ckm_batch_sync(ckm_batch *batch, ckm_stream_t stream);
/* Per-job relative centroid shift of the last step (max |new - old| over
 * max |old|) and iterations done; host arrays of num_jobs entries (either
 * may be NULL).  Synchronises the stream. */
int ckm_batch_status(ckm_batch *batch, float *shifts, uint32_t *iterations, ckm_stream_t stream);
/* Marks jobs active (1) or inactive (0); inactive jobs are skipped by steps. */
int ckm_batch_set_active(ckm_batch *batch, const uint8_t *active, ckm_stream_t stream);
/* Schedule facts: grid, tile points, CTAs per SM, segments. */
int ckm_batch_info(const ckm_batch *batch, uint32_t *grid, uint32_t *tile_points, uint32_t *ctas_per_sm,
                   uint32_t *segments);
int ckm_batch_destroy(ckm_batch *batch);

/* Mixture with chosen laws: centres uniform in [center_a, center_b]
 * (center_dist 0) or normal with mean center_a and standard deviation
 * center_b (1); sigmas uniform (sigma_dist 0) or log-uniform (1) in
 * [sigma_lo, sigma_hi]; component weights equal (dirichlet 0) or
 * Dirichlet(1) (1, at most 12288 blobs).  Point p depends only on (seed, p). */
typedef struct ckm_mixture_spec {
    uint32_t num_features;
    uint32_t num_blobs;
    uint64_t seed;
    int center_dist;
    float center_a, center_b;
    int sigma_dist;
    float sigma_lo, sigma_hi;
    int dirichlet;
} ckm_mixture_spec;
int ckm_generate_mixture_ex_f32(const ckm_mixture_spec *spec, uint64_t num_points, uint64_t first_point,
                                float *points, uint64_t points_stride, ckm_stream_t stream);

/* ---------------------------------------------------------------------- */
/* Host-level run: AbstractKmeans<PointT,LabelT,MassT>::operator()          */
/* (abstract_kmeans.hpp:106-130) through a C ABI, with HOST buffers.  The   */
/* pipeline and per-stage strategies take the reference's .conf names.      */
/* ---------------------------------------------------------------------- */
typedef struct ckm_run_config {
    const char *pipeline;                  /* single_stage | single_stage_buffered |
                                              three_stage | three_stage_buffered */
    const char *fused_strategy;            /* feature_sum | cluster_merge */
    const char *labeling_strategy;         /* unroll_vector */
    const char *mass_update_strategy;      /* global_atomic | part_global | part_local | part_private */
    const char *centroid_update_strategy;  /* feature_sum | feature_sum_pardim | cluster_merge */
    int device;                            /* CUDA device ordinal */
    uint64_t device_budget_bytes;          /* buffered pipelines: device-memory cap (0 = auto) */
    uint64_t chunk_bytes;                  /* buffered pipelines: points bytes per chunk (0 = auto) */
    int converge;                          /* kmeans.converge: stop once the relative centroid shift
                                              (ckm_centroid_shift_*) falls below tolerance */
    double tolerance;                      /* 0 = 1e-4 */
    int spatial_order;                     /* single_stage and three_stage, FP32, d <= 8, k <= 32: run
                                              the iterations on a spatially ordered copy
                                              (ckm_spatial_sort_f32, then the box-pruned
                                              ckm_fused_sorted_f32 / ckm_labeling_sorted_f32); the
                                              last iteration labels the caller's order directly (an
                                              unpermute only when the run stops early).
                                              0 = auto (n >= 2^20, >= 8 iterations, device memory
                                              allows), 1 = whenever the shape allows, -1 = never */
} ckm_run_config;

typedef struct ckm_run_info {
    uint64_t total_time_ns;      /* the reference's TotalTime window (iteration loop) */
    uint64_t h2d_bytes;          /* host -> device bytes moved by the call */
    uint64_t d2h_bytes;          /* device -> host bytes moved by the call */
    uint64_t kernel_launches;    /* kernels this library launched */
    uint32_t iterations;         /* iterations run */
    uint32_t converged;          /* 1 if the run stopped on the convergence test */
    float last_shift;            /* relative centroid shift of the last iteration (converge runs; else 0) */
} ckm_run_info;

/* centroids: in = initial, out = final (k = num_clusters).  masses, labels:
 * out.  info may be NULL. */
int ckm_kmeans_run_f32(const ckm_run_config *config, uint32_t max_iterations,
                       uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                       const float *host_points, float *host_centroids, uint32_t *host_masses,
                       uint32_t *host_labels, ckm_run_info *info);
int ckm_kmeans_run_f64(const ckm_run_config *config, uint32_t max_iterations,
                       uint32_t num_features, uint64_t num_points, uint32_t num_clusters,
                       const double *host_points, double *host_centroids, uint64_t *host_masses,
                       uint64_t *host_labels, ckm_run_info *info);

/* ---------------------------------------------------------------------- */
/* Serving: a stream of independent k-means jobs (continuous batching).    */
/* No counterpart in the reference (one problem per bench invocation).     */
/* Jobs are submitted from any thread with host arrays; a worker thread    */
/* admits them into device memory within a budget, advances every admitted */
/* job by batched launches (ckm_batch_*) in rounds of a few iterations,    */
/* retires each job at its own stopping iteration (relative centroid shift */
/* below the tolerance, or the iteration cap) and copies its results back. */
/* Jobs with n*k*d at or above large_work run one at a time in a second    */
/* lane, on the tensor cores (ckm_tc_fused_f32) when eligible.             */
/* ---------------------------------------------------------------------- */
typedef struct ckm_server ckm_server;

typedef struct ckm_server_options {
    int device;                    /* CUDA device ordinal */
    uint64_t device_budget_bytes;  /* device memory for admitted jobs (0 = half of the free memory) */
    float tolerance;               /* stop once the relative centroid shift is below (0 = 1e-4) */
    uint32_t max_iterations;       /* ... or after this many iterations (0 = 50) */
    uint32_t round_iterations;     /* batched iterations between admissions and retirements (0 = 4) */
    uint64_t large_work;           /* n*k*d from which a job runs in the large-job lane (0 = 2^33) */
} ckm_server_options;

typedef struct ckm_server_job {
    const float *points;           /* host, column-major n x d; must stay valid until the job completes */
    const float *init_centroids;   /* host, column-major k x d */
    float *centroids;              /* host out, k x d */
    uint32_t *masses;              /* host out, k */
    uint32_t *labels;              /* host out, n; NULL: labels are not returned */
    uint64_t num_points;
    uint32_t num_features;
    uint32_t num_clusters;
    uint64_t tag;                  /* the caller's identifier, returned with the result */
} ckm_server_job;

typedef struct ckm_server_result {
    uint64_t tag;
    int status;                    /* CKM_OK, or why the job failed */
    uint32_t iterations;
    uint32_t converged;            /* 1: stopped on the tolerance; 0: on the iteration cap */
    float shift;                   /* relative centroid shift of the last iteration */
    uint32_t lane;                 /* 0: batched lane; 1: large-job lane on the tensor cores; 2: large-job lane, SIMT */
    uint64_t first_round;          /* batched lane: the first round (1, 2, ...) the job ran in; 0 otherwise */
    uint64_t last_round;           /* batched lane: the round in which it stopped; 0 otherwise */
    uint64_t latency_ns;           /* submit -> results in the caller's host arrays */
    char error[128];               /* why the job failed (empty when status is CKM_OK) */
} ckm_server_result;

int ckm_server_create(const ckm_server_options *options, ckm_server **out);
/* Queues a job (copies the descriptor, not the arrays); thread-safe. */
int ckm_server_submit(ckm_server *server, const ckm_server_job *job);
/* Results of the jobs completed since the last poll, oldest first (at most
 * max_results; *count receives how many); never blocks. */
int ckm_server_poll(ckm_server *server, ckm_server_result *results, uint32_t max_results, uint32_t *count);
/* Blocks until every job submitted so far has completed. */
int ckm_server_drain(ckm_server *server);
/* Cumulative counters of the batched lane since creation. */
typedef struct ckm_server_stats {
    uint64_t rounds;               /* batched rounds run */
    uint64_t job_rounds;           /* sum over rounds of the jobs in the round */
    uint64_t busy_ns;              /* wall time of the rounds (schedule, steps, status, retirement) */
    uint64_t steps_gpu_ns;         /* device time of the rounds' batched launches (CUDA events) */
    uint64_t admit_ns;             /* host time spent admitting jobs (allocation, copies enqueued) */
    uint64_t retire_ns;            /* host time spent copying results back and releasing jobs */
    uint64_t jobs_admitted;
    uint64_t jobs_completed;
} ckm_server_stats;
int ckm_server_stats_get(ckm_server *server, ckm_server_stats *stats);
/* Drains, stops the worker threads and frees everything. */
int ckm_server_destroy(ckm_server *server);

/* Host <-> device link probe (the roofline of the buffered pipelines, whose
 * points cross this link every iteration).  Times `repeat` back-to-back
 * copies of chunk_bytes between host memory (pinned != 0: page-locked,
 * else pageable) and one device buffer, to the device (to_device != 0) or
 * back, over `trials` timed trials after one warm-up; reports the best and
 * mean GB/s (mean_gbs may be NULL).  device < 0 keeps the current device.
 * It allocates its own host and device buffers.  Replaces the measurement of
 * transfer_bench.cpp (buffer sizes up to --max-size pushed through the
 * buffer cache, --repeat times). */
int ckm_transfer_probe(int device, uint64_t chunk_bytes, uint32_t repeat, int pinned, int to_device,
                       uint32_t trials, double *best_gbs, double *mean_gbs);

#ifdef __cplusplus
}
#endif

#endif /* CKM_H */
