// Single-stage (fused) strategy: KmeansSingleStage
// (kmeans_single_stage.hpp:31-381).  Uploads points and centroids, then runs
// the iteration loop inside the TotalTime window and copies centroids,
// labels and masses back.  Where the reference enqueues fill, fill, fused,
// 2x reduce, 2x add and divide per iteration (kmeans_single_stage.hpp:97-144,
// fused_feature_sum.hpp:369-439), each iteration here is ONE launch of the
// fused kernel in FINALIZE mode; with graphs enabled the whole loop is one
// CUDA graph.
#pragma once

#include <algorithm>
#include <type_traits>

#include "abstract_kmeans.hpp"
#include "factories.hpp"
#include "timer.hpp"

namespace Clustering {

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class KmeansSingleStage : public AbstractKmeans<PointT, LabelT, MassT, ColMajor> {
public:
    using FusedFunction = typename FusedFactory<PointT, LabelT, MassT, ColMajor>::FusedFunction;

    void run() override {
        if (!queue_.valid()) queue_ = Stream::create();
        const size_t d = this->num_features, n = this->num_points, k = this->num_clusters;

        points_.resize(n * d);
        centroids_.resize(k * d);
        new_centroids_.resize(k * d);
        labels_.resize(n);
        masses_.resize(k);
        {
            auto& dp = this->measurement->add_datapoint().set_name("PointsH2D");
            Event& ev = dp.add_event(queue_);
            points_.upload_async(this->in_points(), n * d, queue_);
            ev.record_end(queue_);
        }
        {
            auto& dp = this->measurement->add_datapoint().set_name("CentroidsH2D");
            Event& ev = dp.add_event(queue_);
            centroids_.upload_async(this->io_centroids(), k * d, queue_);
            ev.record_end(queue_);
        }
        new_centroids_.fill_zero_async(queue_);
        labels_.fill_zero_async(queue_);
        masses_.fill_zero_async(queue_);
        engine_.reserve((uint32_t)d, (uint32_t)k, queue_);
        if (this->centroids_initializer) this->centroids_initializer(points_, centroids_);
        queue_.finish();
        this->measurement->set_origin(queue_);

        Timer::Timer total_timer;
        total_timer.start();
        this->reset_progress();
        // spatial order: the iterations run on a Z-ordered copy of the points
        // with per-warp box pruning (same labels per point, mapped back to
        // the caller's order after the loop); the sort is inside the window
        const bool spatial = use_spatial_order(d, n, k);
        const PointT* iter_points = points_.data();
        if (spatial) {
            auto& dp = this->measurement->add_datapoint().set_name("SpatialSort");
            Event& ev = dp.add_event(queue_);
            sorted_points_.resize(n * d);
            // the permutation is only needed to bring the labels back when
            // the run can stop early (the last iteration of a full run labels
            // the caller's order directly)
            if (this->converge) perm_.resize(n);
            sort_ws_.resize(ckm_spatial_sort_workspace_bytes(n, (uint32_t)d));
            ckm_check(ckm_spatial_sort_f32((uint32_t)d, n, reinterpret_cast<const float*>(points_.data()),
                                           reinterpret_cast<float*>(sorted_points_.data()),
                                           this->converge ? perm_.data() : nullptr,
                                           sort_ws_.data(), sort_ws_.size(), queue_.get()),
                      "SpatialSort");
            ev.record_end(queue_);
            iter_points = sorted_points_.data();
        }
        bool labels_sorted = false;  // labels_ holds the sorted set's order
        for (uint32_t iteration = 0; iteration < this->max_iterations; ++iteration) {
            // the last iteration of a full run labels the caller's order
            // directly (the same labels per point), so no unpermute is needed
            if (spatial && iteration + 1 < this->max_iterations) {
                labels_sorted = true;
                auto& dp = this->measurement->add_datapoint((int)iteration).set_name("FusedFeatureSumSorted");
                Event& ev = dp.add_event(queue_);
                Scratch& sc = engine_.scratch();
                sc.reserve((uint32_t)d, (uint32_t)k, queue_);
                // a run that cannot stop early reads none of these labels
                // (its last iteration labels the caller's order): skip them
                ckm_check(ckm_fused_sorted_f32((uint32_t)d, n, (uint32_t)k,
                                               reinterpret_cast<const float*>(iter_points),
                                               reinterpret_cast<const float*>(centroids_.data()),
                                               reinterpret_cast<float*>(new_centroids_.data()),
                                               this->converge ? reinterpret_cast<uint32_t*>(labels_.data())
                                                              : nullptr,
                                               reinterpret_cast<uint32_t*>(masses_.data()), sc.data(), sc.bytes(),
                                               CKM_MODE_FINALIZE, queue_.get()),
                          "FusedFeatureSumSorted");
                ev.record_end(queue_);
            } else {
                labels_sorted = false;
                engine_.launch(queue_, d, n, k, points_.data(), centroids_.data(), new_centroids_.data(),
                               labels_.data(), masses_.data(), CKM_MODE_FINALIZE,
                               this->measurement->add_datapoint((int)iteration), WaitList());
            }
            centroids_.swap(new_centroids_);
            if (this->after_iteration(iteration, probe_, (uint32_t)d, (uint32_t)k, new_centroids_.data(),
                                      centroids_.data(), queue_))
                break;
        }
        if (labels_sorted) {
            // stopped early on the convergence test: labels back to the
            // caller's order
            labels_out_.resize(n);
            ckm_check(ckm_unpermute_u32(n, perm_.data(), reinterpret_cast<const uint32_t*>(labels_.data()),
                                        reinterpret_cast<uint32_t*>(labels_out_.data()), queue_.get()),
                      "UnpermuteLabels");
        }
        queue_.finish();
        uint64_t total_time = total_timer.stop<std::chrono::nanoseconds>();
        this->measurement->add_datapoint().set_name("TotalTime").add_value() = total_time;
        last_total_ns_ = total_time;
        last_spatial_ = spatial;

        download("CentroidsD2H", centroids_, this->io_centroids(), k * d);
        download("LabelsD2H", labels_sorted ? labels_out_ : labels_, this->out_labels(), n);
        download("MassesD2H", masses_, this->out_masses(), k);
        queue_.finish();
        h2d_bytes_ = (n * d + k * d) * sizeof(PointT);
        d2h_bytes_ = k * d * sizeof(PointT) + n * sizeof(LabelT) + k * sizeof(MassT);
    }

    void set_fused(FusedConfiguration config) {
        FusedFactory<PointT, LabelT, MassT, ColMajor> factory;
        engine_ = factory.create_engine(config, *this->measurement);
        f_fused = engine_;
    }

    void set_queue(Stream q) {
        queue_ = q;
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, q.device()) == cudaSuccess) {
            this->measurement->set_parameter("FusedPlatform", "CUDA");
            this->measurement->set_parameter("FusedDevice", p.name);
        }
    }

    // Spatial order of the iterations: 0 = auto (FP32, d <= 8, k <= 32,
    // n >= 2^20, >= 8 iterations, enough free device memory), 1 = whenever
    // the shape allows, -1 = never.
    void set_spatial_order(int mode) { spatial_mode_ = mode; }
    bool used_spatial_order() const { return last_spatial_; }

    uint64_t last_total_ns() const { return last_total_ns_; }
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }

    FusedFunction f_fused;

private:
    template <typename T>
    void download(const char* name, const DeviceVector<T>& src, T* dst, size_t count) {
        auto& dp = this->measurement->add_datapoint().set_name(name);
        Event& ev = dp.add_event(queue_);
        src.download_async(dst, count, queue_);
        ev.record_end(queue_);
    }

    bool use_spatial_order(size_t d, size_t n, size_t k) const {
        return spatial_order_eligible<PointT, LabelT, MassT, ColMajor>(spatial_mode_, d, n, k, this->max_iterations);
    }

    FusedLloyd<PointT, LabelT, MassT> engine_;
    ConvergenceProbe<PointT, LabelT, MassT> probe_;
    Stream queue_;
    DeviceVector<PointT> points_, centroids_, new_centroids_, sorted_points_;
    DeviceVector<LabelT> labels_, labels_out_;
    DeviceVector<MassT> masses_;
    DeviceVector<uint32_t> perm_;
    DeviceVector<unsigned char> sort_ws_;
    int spatial_mode_ = 0;
    bool last_spatial_ = false;
    uint64_t last_total_ns_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
};

}  // namespace Clustering
