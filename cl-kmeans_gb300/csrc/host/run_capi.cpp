// ckm_kmeans_run_*: the host-level call (AbstractKmeans::operator(),
// abstract_kmeans.hpp:106-130) exported through the C ABI.  Builds the
// strategy the reference's bench.cpp:319-404 would build for the pipeline
// name, runs it over the caller's host arrays and reports the TotalTime
// window and the bytes moved.  Exceptions never cross the ABI: unknown
// strategy names map to CKM_ERR_UNKNOWN_STRATEGY, CUDA failures to
// CKM_ERR_CUDA.
#include <cstring>
#include <stdexcept>
#include <string>

#include "../ckm_internal.h"
#include "kmeans_buffered.hpp"
#include "kmeans_single_stage.hpp"
#include "kmeans_three_stage.hpp"

namespace Clustering {

void ckm_check(int status, const char* where) {
    if (status != CKM_OK) {
        std::string msg = std::string(where) + ": " + ckm_status_string(status);
        const char* detail = ckm_last_error();
        if (detail && *detail) msg += std::string(" (") + detail + ")";
        throw KernelError(status, msg);
    }
}

}  // namespace Clustering

namespace {

using namespace Clustering;

const char* or_default(const char* s, const char* d) { return (s && *s) ? s : d; }

template <typename P, typename L, typename M>
int run_impl(const ckm_run_config* cfg, uint32_t iters, uint32_t d, uint64_t n, uint32_t k, const P* points,
             P* centroids, M* masses, L* labels, ckm_run_info* info) {
    if (!cfg) return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "config is NULL");
    if (d == 0 || k == 0) return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "num_features and num_clusters must be >= 1");
    if (n > 0 && (!points || !labels)) return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "points/labels NULL");
    if (!centroids || !masses) return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "centroids/masses NULL");
    const std::string pipeline = or_default(cfg->pipeline, "single_stage");
    // names are checked before any device work, as the reference's factories
    // reject an unknown strategy when they are configured
    const bool single = pipeline == "single_stage" || pipeline == "single_stage_buffered";
    const bool three = pipeline == "three_stage" || pipeline == "three_stage_buffered";
    if (!single && !three) return ckm::fail(CKM_ERR_UNKNOWN_STRATEGY, "unknown pipeline '" + pipeline + "'");
    const std::string fused = or_default(cfg->fused_strategy, "feature_sum");
    const std::string labeling = or_default(cfg->labeling_strategy, "unroll_vector");
    const std::string mass = or_default(cfg->mass_update_strategy, "part_local");
    const std::string update = or_default(cfg->centroid_update_strategy, "feature_sum");
    const char* bad = nullptr;
    if (single && !FusedFactory<P, L, M, true>::known(fused)) bad = fused.c_str();
    if (three && !LabelingFactory<P, L, true>::known(labeling)) bad = labeling.c_str();
    if (three && !MassUpdateFactory<L, M>::known(mass)) bad = mass.c_str();
    if (three && !CentroidUpdateFactory<P, L, M, true>::known(update)) bad = update.c_str();
    if (bad) return ckm::fail(CKM_ERR_UNKNOWN_STRATEGY, std::string("unknown strategy: ") + bad);
    const uint64_t launches0 = ckm::launch_count();
    try {
        if (cfg->device >= 0) cuda_check(cudaSetDevice(cfg->device), "cudaSetDevice");
        uint64_t total_ns = 0, h2d = 0, d2h = 0;
        uint32_t done = 0, conv = 0;
        float shift = 0.0f;
        if (pipeline == "single_stage") {
            KmeansSingleStage<P, L, M> s;
            FusedConfiguration fc;
            fc.strategy = or_default(cfg->fused_strategy, "feature_sum");
            s.set_fused(fc);
            s.set_converge(cfg->converge != 0);
            s.set_tolerance(cfg->tolerance);
            s.set_spatial_order(cfg->spatial_order);
            s.run_raw(iters, d, n, k, points, centroids, masses, labels);
            done = (uint32_t)s.iterations_done();
            conv = s.did_converge() ? 1u : 0u;
            shift = s.last_shift();
            total_ns = s.last_total_ns();
            h2d = s.h2d_bytes();
            d2h = s.d2h_bytes();
        } else if (pipeline == "three_stage") {
            KmeansThreeStage<P, L, M> s;
            LabelingConfiguration lc;
            lc.strategy = or_default(cfg->labeling_strategy, "unroll_vector");
            MassUpdateConfiguration mc;
            mc.strategy = or_default(cfg->mass_update_strategy, "part_local");
            CentroidUpdateConfiguration cc;
            cc.strategy = or_default(cfg->centroid_update_strategy, "feature_sum");
            s.set_labeler(lc);
            s.set_mass_updater(mc);
            s.set_centroid_updater(cc);
            s.set_converge(cfg->converge != 0);
            s.set_tolerance(cfg->tolerance);
            s.set_spatial_order(cfg->spatial_order);
            s.run_raw(iters, d, n, k, points, centroids, masses, labels);
            done = (uint32_t)s.iterations_done();
            conv = s.did_converge() ? 1u : 0u;
            shift = s.last_shift();
            total_ns = s.last_total_ns();
            h2d = s.h2d_bytes();
            d2h = s.d2h_bytes();
        } else if (pipeline == "single_stage_buffered" || pipeline == "three_stage_buffered") {
            BufferedOptions opt;
            opt.device_budget_bytes = cfg->device_budget_bytes;
            opt.chunk_bytes = cfg->chunk_bytes;
            if (pipeline == "single_stage_buffered") {
                KmeansSingleStageBuffered<P, L, M> s;
                FusedConfiguration fc;
                fc.strategy = or_default(cfg->fused_strategy, "feature_sum");
                s.set_fused(fc);
                s.set_options(opt);
                s.set_converge(cfg->converge != 0);
                s.set_tolerance(cfg->tolerance);
                s.run_raw(iters, d, n, k, points, centroids, masses, labels);
                done = (uint32_t)s.iterations_done();
                conv = s.did_converge() ? 1u : 0u;
                shift = s.last_shift();
                total_ns = s.last_total_ns();
                h2d = s.h2d_bytes();
                d2h = s.d2h_bytes();
            } else {
                KmeansThreeStageBuffered<P, L, M> s;
                LabelingConfiguration lc;
                lc.strategy = or_default(cfg->labeling_strategy, "unroll_vector");
                MassUpdateConfiguration mc;
                mc.strategy = or_default(cfg->mass_update_strategy, "part_local");
                CentroidUpdateConfiguration cc;
                cc.strategy = or_default(cfg->centroid_update_strategy, "feature_sum");
                s.set_labeler(lc);
                s.set_mass_updater(mc);
                s.set_centroid_updater(cc);
                s.set_options(opt);
                s.set_converge(cfg->converge != 0);
                s.set_tolerance(cfg->tolerance);
                s.run_raw(iters, d, n, k, points, centroids, masses, labels);
                done = (uint32_t)s.iterations_done();
                conv = s.did_converge() ? 1u : 0u;
                shift = s.last_shift();
                total_ns = s.last_total_ns();
                h2d = s.h2d_bytes();
                d2h = s.d2h_bytes();
            }
        } else {
            return ckm::fail(CKM_ERR_UNKNOWN_STRATEGY, "unknown pipeline '" + pipeline + "'");
        }
        if (info) {
            info->total_time_ns = total_ns;
            info->h2d_bytes = h2d;
            info->d2h_bytes = d2h;
            info->kernel_launches = ckm::launch_count() - launches0;
            info->iterations = done;
            info->converged = conv;
            info->last_shift = shift;
        }
        return CKM_OK;
    } catch (const KernelError& e) {
        return ckm::fail(e.status, e.what());
    } catch (const BudgetError& e) {
        return ckm::fail(CKM_ERR_BUDGET, e.what());
    } catch (const CudaError& e) {
        return ckm::fail(CKM_ERR_CUDA, e.what());
    } catch (const std::invalid_argument& e) {
        return ckm::fail(CKM_ERR_UNKNOWN_STRATEGY, std::string("unknown strategy: ") + e.what());
    } catch (const std::bad_alloc&) {
        return ckm::fail(CKM_ERR_ALLOC, "host allocation failed");
    } catch (const std::exception& e) {
        return ckm::fail(CKM_ERR_INVALID_ARGUMENT, e.what());
    }
}

}  // namespace

extern "C" {

int ckm_kmeans_run_f32(const ckm_run_config* config, uint32_t max_iterations, uint32_t num_features,
                       uint64_t num_points, uint32_t num_clusters, const float* host_points, float* host_centroids,
                       uint32_t* host_masses, uint32_t* host_labels, ckm_run_info* info) {
    return run_impl<float, uint32_t, uint32_t>(config, max_iterations, num_features, num_points, num_clusters,
                                               host_points, host_centroids, host_masses, host_labels, info);
}

int ckm_kmeans_run_f64(const ckm_run_config* config, uint32_t max_iterations, uint32_t num_features,
                       uint64_t num_points, uint32_t num_clusters, const double* host_points,
                       double* host_centroids, uint64_t* host_masses, uint64_t* host_labels, ckm_run_info* info) {
    return run_impl<double, uint64_t, uint64_t>(config, max_iterations, num_features, num_points, num_clusters,
                                                host_points, host_centroids, host_masses, host_labels, info);
}

}  // extern "C"
