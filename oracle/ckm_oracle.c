/*
 * ckm_oracle.c -- CPU restatement of the reference's Lloyd k-means iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke
 * entry point and bench.py's CPU-baseline / reference legs may call it.  The
 * product path (the CUDA library) never links, loads or calls it.
 *
 * Parity pin: every routine here is checked bit-for-bit against the
 * reference's own KmeansNaive (kmeans_naive.cpp), compiled unchanged by
 * oracle/build_ref.sh into oracle/_ref/, and against golden fixtures made from
 * that build (tests/golden/).
 *
 * Layouts (reference convention, lloyd_fused_feature_sum.cl:77-79, 200, 230):
 *   points     column-major  P[f * n + p]
 *   centroids  column-major  C[f * k + c]
 *   labels     one per point, masses one per cluster
 *
 * Compile with -ffp-contract=off: the distance uses explicit fma (the form
 * GCC contracts `distance += t * t` into under the reference's
 * -ffp-contract=fast, and the form the OpenCL kernels spell out), and the
 * Kahan sums must not be fused.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* FP32 labeling: kmeans_naive.cpp:48-69 (and lloyd_labeling_vp_clcp.cl,      */
/* lloyd_fused_feature_sum.cl:209-239).  min starts at FLT_MAX, label at 0,  */
/* strict '<' so the lowest index wins a tie and NaN never wins.              */
/* ------------------------------------------------------------------------ */
static inline uint32_t label_one_f32(const float *P, uint64_t n, uint32_t d,
                                     uint32_t k, uint64_t p, const float *C) {
    float min_distance = FLT_MAX;
    uint32_t min_centroid = 0;
    for (uint32_t c = 0; c < k; ++c) {
        float distance = 0.0f;
        for (uint32_t f = 0; f < d; ++f) {
            float t = P[(uint64_t)f * n + p] - C[(uint64_t)f * k + c];
            distance = fmaf(t, t, distance);
        }
        if (distance < min_distance) {
            min_distance = distance;
            min_centroid = c;
        }
    }
    return min_centroid;
}

static inline uint64_t label_one_f64(const double *P, uint64_t n, uint32_t d,
                                     uint32_t k, uint64_t p, const double *C) {
    double min_distance = DBL_MAX;
    uint64_t min_centroid = 0;
    for (uint32_t c = 0; c < k; ++c) {
        double distance = 0.0;
        for (uint32_t f = 0; f < d; ++f) {
            double t = P[(uint64_t)f * n + p] - C[(uint64_t)f * k + c];
            distance = fma(t, t, distance);
        }
        if (distance < min_distance) {
            min_distance = distance;
            min_centroid = c;
        }
    }
    return min_centroid;
}

void ckm_oracle_label_f32(const float *P, uint64_t n, uint32_t d, uint32_t k,
                          const float *C, uint32_t *labels) {
    for (uint64_t p = 0; p < n; ++p) labels[p] = label_one_f32(P, n, d, k, p, C);
}

void ckm_oracle_label_f64(const double *P, uint64_t n, uint32_t d, uint32_t k,
                          const double *C, uint64_t *labels) {
    for (uint64_t p = 0; p < n; ++p) labels[p] = label_one_f64(P, n, d, k, p, C);
}

/* ------------------------------------------------------------------------ */
/* Mass histogram: kmeans_naive.cpp:74-79 (histogram_*.cl): exact counts.     */
/* Accumulates into masses (the MassUpdate functor contract, caller zeroes). */
/* ------------------------------------------------------------------------ */
void ckm_oracle_mass_u32(const uint32_t *labels, uint64_t n, uint32_t k,
                         uint32_t *masses) {
    for (uint64_t p = 0; p < n; ++p)
        if (labels[p] < k) masses[labels[p]] += 1;
}

/* ------------------------------------------------------------------------ */
/* Centroid update, FP32 Kahan: kmeans_naive.cpp:70-100.                      */
/* Writes the new centroids (sum / mass, 0/0 -> NaN) and masses.              */
/* ------------------------------------------------------------------------ */
void ckm_oracle_update_f32(const float *P, uint64_t n, uint32_t d, uint32_t k,
                           const uint32_t *labels, float *C, uint32_t *masses) {
    float *comp = (float *)calloc((size_t)k * d, sizeof(float));
    memset(masses, 0, sizeof(uint32_t) * k);
    memset(C, 0, sizeof(float) * (size_t)k * d);
    for (uint64_t p = 0; p < n; ++p) {
        uint32_t c = labels[p];
        masses[c] += 1;
        for (uint32_t f = 0; f < d; ++f) {
            float point = P[(uint64_t)f * n + p];
            float *cp = &comp[(uint64_t)f * k + c];
            float *sum = &C[(uint64_t)f * k + c];
            float y = point - *cp;
            float t = *sum + y;
            *cp = (t - *sum) - y;
            *sum = t;
        }
    }
    for (uint32_t f = 0; f < d; ++f)
        for (uint32_t c = 0; c < k; ++c)
            C[(uint64_t)f * k + c] = C[(uint64_t)f * k + c] / (float)masses[c];
    free(comp);
}

void ckm_oracle_update_f64(const double *P, uint64_t n, uint32_t d, uint32_t k,
                           const uint64_t *labels, double *C, uint64_t *masses) {
    double *comp = (double *)calloc((size_t)k * d, sizeof(double));
    memset(masses, 0, sizeof(uint64_t) * k);
    memset(C, 0, sizeof(double) * (size_t)k * d);
    for (uint64_t p = 0; p < n; ++p) {
        uint64_t c = labels[p];
        masses[c] += 1;
        for (uint32_t f = 0; f < d; ++f) {
            double point = P[(uint64_t)f * n + p];
            double *cp = &comp[(uint64_t)f * k + c];
            double *sum = &C[(uint64_t)f * k + c];
            double y = point - *cp;
            double t = *sum + y;
            *cp = (t - *sum) - y;
            *sum = t;
        }
    }
    for (uint32_t f = 0; f < d; ++f)
        for (uint32_t c = 0; c < k; ++c)
            C[(uint64_t)f * k + c] = C[(uint64_t)f * k + c] / (double)masses[c];
    free(comp);
}

/* ------------------------------------------------------------------------ */
/* Whole run: kmeans_naive.cpp:31-106 (no early stop, did_changes unused).   */
/* ------------------------------------------------------------------------ */
void ckm_oracle_lloyd_f32(const float *P, uint64_t n, uint32_t d, uint32_t k,
                          uint32_t iterations, float *C, uint32_t *masses,
                          uint32_t *labels) {
    for (uint32_t it = 0; it < iterations; ++it) {
        ckm_oracle_label_f32(P, n, d, k, C, labels);
        ckm_oracle_update_f32(P, n, d, k, labels, C, masses);
    }
}

void ckm_oracle_lloyd_f64(const double *P, uint64_t n, uint32_t d, uint32_t k,
                          uint32_t iterations, double *C, uint64_t *masses,
                          uint64_t *labels) {
    for (uint32_t it = 0; it < iterations; ++it) {
        ckm_oracle_label_f64(P, n, d, k, C, labels);
        ckm_oracle_update_f64(P, n, d, k, labels, C, masses);
    }
}

/* ------------------------------------------------------------------------ */
/* first_x initialiser: kmeans_initializer.cpp:29-39 (C[f,c] = P[c % n, f]).  */
/* ------------------------------------------------------------------------ */
void ckm_oracle_first_x_f32(const float *P, uint64_t n, uint32_t d, uint32_t k,
                            float *C) {
    for (uint32_t f = 0; f < d; ++f)
        for (uint32_t c = 0; c < k; ++c)
            C[(uint64_t)f * k + c] = P[(uint64_t)f * n + (c % n)];
}

/* ------------------------------------------------------------------------ */
/* FP64 adjudication oracle (not in the reference; the FP64 restatement of    */
/* kmeans_naive.cpp:48-69 used to judge near-ties).  For FP32 points and FP32 */
/* centroids it returns, per point, the FP64 argmin and the FP64 gap between  */
/* the best and second-best squared distance.                                 */
/* ------------------------------------------------------------------------ */
void ckm_oracle_label_gap_f64(const float *P, uint64_t n, uint32_t d, uint32_t k,
                              const float *C, uint32_t *labels, double *gap,
                              double *best) {
    for (uint64_t p = 0; p < n; ++p) {
        double b0 = DBL_MAX, b1 = DBL_MAX;
        uint32_t l0 = 0;
        for (uint32_t c = 0; c < k; ++c) {
            double dist = 0.0;
            for (uint32_t f = 0; f < d; ++f) {
                double t = (double)P[(uint64_t)f * n + p] - (double)C[(uint64_t)f * k + c];
                dist = fma(t, t, dist);
            }
            if (dist < b0) {
                b1 = b0;
                b0 = dist;
                l0 = c;
            } else if (dist < b1) {
                b1 = dist;
            }
        }
        labels[p] = l0;
        gap[p] = b1 - b0;
        best[p] = b0;
    }
}

/* FP64 Lloyd on FP32 points with FP64 centroids (the spec FP64 oracle):
 * same argmin rule, plain FP64 sums in point order. */
void ckm_oracle_lloyd_fp64_of_f32(const float *P, uint64_t n, uint32_t d,
                                  uint32_t k, uint32_t iterations, double *C,
                                  uint64_t *masses, uint32_t *labels) {
    double *sums = (double *)malloc(sizeof(double) * (size_t)k * d);
    for (uint32_t it = 0; it < iterations; ++it) {
        for (uint64_t p = 0; p < n; ++p) {
            double min_distance = DBL_MAX;
            uint32_t min_centroid = 0;
            for (uint32_t c = 0; c < k; ++c) {
                double dist = 0.0;
                for (uint32_t f = 0; f < d; ++f) {
                    double t = (double)P[(uint64_t)f * n + p] - C[(uint64_t)f * k + c];
                    dist = fma(t, t, dist);
                }
                if (dist < min_distance) {
                    min_distance = dist;
                    min_centroid = c;
                }
            }
            labels[p] = min_centroid;
        }
        memset(sums, 0, sizeof(double) * (size_t)k * d);
        memset(masses, 0, sizeof(uint64_t) * k);
        for (uint64_t p = 0; p < n; ++p) {
            uint32_t c = labels[p];
            masses[c] += 1;
            for (uint32_t f = 0; f < d; ++f)
                sums[(uint64_t)f * k + c] += (double)P[(uint64_t)f * n + p];
        }
        for (uint32_t f = 0; f < d; ++f)
            for (uint32_t c = 0; c < k; ++c)
                C[(uint64_t)f * k + c] = sums[(uint64_t)f * k + c] / (double)masses[c];
    }
    free(sums);
}

/* FP64 per-cluster sums of FP32 points for given labels (exact enough to
 * bound the GPU's FP64-merged sums; column-major like the centroids). */
void ckm_oracle_sums_f64(const float *P, uint64_t n, uint32_t d, uint32_t k,
                         const uint32_t *labels, double *sums, uint64_t *masses) {
    memset(sums, 0, sizeof(double) * (size_t)k * d);
    memset(masses, 0, sizeof(uint64_t) * k);
    for (uint64_t p = 0; p < n; ++p) {
        uint32_t c = labels[p];
        if (c >= k) continue;
        masses[c] += 1;
        for (uint32_t f = 0; f < d; ++f)
            sums[(uint64_t)f * k + c] += (double)P[(uint64_t)f * n + p];
    }
}

/* ------------------------------------------------------------------------ */
/* partition_matrix restatement: buffer_helper.cpp:16-87.  Re-lays a          */
/* column-major matrix of `size` bytes and `num_dims` columns into chunks of  */
/* `buffer_size` bytes, each chunk column-major over its own point slice.     */
/* Returns the chunk count, or -1 on a dimension mismatch.                    */
/* ------------------------------------------------------------------------ */
int ckm_oracle_partition_matrix(const void *src, void *dst, size_t size,
                                size_t num_dims, size_t buffer_size) {
    if (num_dims == 0 || size % num_dims != 0 || buffer_size % num_dims != 0)
        return -1;
    size_t dim_size = size / num_dims;
    size_t buf_dim_size = buffer_size / num_dims;
    size_t num_bufs = (size + buffer_size - 1) / buffer_size;
    const char *s = (const char *)src;
    char *o = (char *)dst;
    for (size_t b = 0; b < num_bufs; ++b) {
        for (size_t v = 0; v < num_dims; ++v) {
            size_t real = (buf_dim_size * (b + 1) > dim_size)
                              ? dim_size - b * buf_dim_size
                              : buf_dim_size;
            memcpy(&o[b * buffer_size + v * real], &s[v * dim_size + b * buf_dim_size],
                   real);
        }
    }
    return (int)num_bufs;
}

/* ------------------------------------------------------------------------ */
/* Threaded FP32 Lloyd for the timed CPU legs.  Labeling is per point, so it  */
/* is bit-identical to the serial restatement.  Each thread keeps Kahan       */
/* partials over its contiguous point range; partials merge in thread order,  */
/* so the centroids differ from the serial Kahan order only by rounding.      */
/* ------------------------------------------------------------------------ */
typedef struct {
    const float *P;
    uint64_t n, lo, hi;
    uint32_t d, k;
    const float *C;
    uint32_t *labels;
    float *sum, *comp;
    uint32_t *mass;
} mt_job;

static void *mt_label_and_sum(void *arg) {
    mt_job *j = (mt_job *)arg;
    memset(j->sum, 0, sizeof(float) * (size_t)j->k * j->d);
    memset(j->comp, 0, sizeof(float) * (size_t)j->k * j->d);
    memset(j->mass, 0, sizeof(uint32_t) * j->k);
    for (uint64_t p = j->lo; p < j->hi; ++p) {
        uint32_t c = label_one_f32(j->P, j->n, j->d, j->k, p, j->C);
        j->labels[p] = c;
        j->mass[c] += 1;
        for (uint32_t f = 0; f < j->d; ++f) {
            float point = j->P[(uint64_t)f * j->n + p];
            float *cp = &j->comp[(uint64_t)f * j->k + c];
            float *s = &j->sum[(uint64_t)f * j->k + c];
            float y = point - *cp;
            float t = *s + y;
            *cp = (t - *s) - y;
            *s = t;
        }
    }
    return NULL;
}

int ckm_oracle_lloyd_f32_mt(const float *P, uint64_t n, uint32_t d, uint32_t k,
                            uint32_t iterations, float *C, uint32_t *masses,
                            uint32_t *labels, int threads) {
    if (threads < 1) threads = 1;
    if ((uint64_t)threads > n) threads = (int)(n ? n : 1);
    mt_job *jobs = (mt_job *)calloc((size_t)threads, sizeof(mt_job));
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    float *bufs = (float *)malloc(sizeof(float) * (size_t)threads * 2 * k * d);
    uint32_t *mbuf = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)threads * k);
    if (!jobs || !tid || !bufs || !mbuf) return -1;
    for (uint32_t it = 0; it < iterations; ++it) {
        for (int t = 0; t < threads; ++t) {
            mt_job *j = &jobs[t];
            j->P = P; j->n = n; j->d = d; j->k = k; j->C = C; j->labels = labels;
            j->lo = n * (uint64_t)t / (uint64_t)threads;
            j->hi = n * (uint64_t)(t + 1) / (uint64_t)threads;
            j->sum = bufs + (size_t)t * 2 * k * d;
            j->comp = j->sum + (size_t)k * d;
            j->mass = mbuf + (size_t)t * k;
            if (t > 0) pthread_create(&tid[t], NULL, mt_label_and_sum, j);
        }
        mt_label_and_sum(&jobs[0]);
        for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
        memset(masses, 0, sizeof(uint32_t) * k);
        for (uint64_t e = 0; e < (uint64_t)k * d; ++e) {
            float s = 0.0f, cmp = 0.0f;
            for (int t = 0; t < threads; ++t) {
                float y = jobs[t].sum[e] - cmp;
                float tt = s + y;
                cmp = (tt - s) - y;
                s = tt;
            }
            C[e] = s;
        }
        for (int t = 0; t < threads; ++t)
            for (uint32_t c = 0; c < k; ++c) masses[c] += jobs[t].mass[c];
        for (uint32_t f = 0; f < d; ++f)
            for (uint32_t c = 0; c < k; ++c)
                C[(uint64_t)f * k + c] = C[(uint64_t)f * k + c] / (float)masses[c];
    }
    free(jobs); free(tid); free(bufs); free(mbuf);
    return 0;
}
