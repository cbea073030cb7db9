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
        for (uint32_t iteration = 0; iteration < this->max_iterations; ++iteration) {
            engine_.launch(queue_, d, n, k, points_.data(), centroids_.data(), new_centroids_.data(),
                           labels_.data(), masses_.data(), CKM_MODE_FINALIZE,
                           this->measurement->add_datapoint((int)iteration), WaitList());
            centroids_.swap(new_centroids_);
            if (this->after_iteration(iteration, probe_, (uint32_t)d, (uint32_t)k, new_centroids_.data(),
                                      centroids_.data(), queue_))
                break;
        }
        queue_.finish();
        uint64_t total_time = total_timer.stop<std::chrono::nanoseconds>();
        this->measurement->add_datapoint().set_name("TotalTime").add_value() = total_time;
        last_total_ns_ = total_time;

        download("CentroidsD2H", centroids_, this->io_centroids(), k * d);
        download("LabelsD2H", labels_, this->out_labels(), n);
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

    FusedLloyd<PointT, LabelT, MassT> engine_;
    ConvergenceProbe<PointT, LabelT, MassT> probe_;
    Stream queue_;
    DeviceVector<PointT> points_, centroids_, new_centroids_;
    DeviceVector<LabelT> labels_;
    DeviceVector<MassT> masses_;
    uint64_t last_total_ns_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
};

}  // namespace Clustering
