// Three-stage strategy: KmeansThreeStage (kmeans_three_stage.hpp:30-335).
// Per iteration: labeling -> fill masses -> mass update -> centroid update ->
// divide, on up to three queues (one per stage, as the reference's
// set_*_queue setters allow).  The points are read twice per iteration
// (labeling and centroid update), which is the traffic the fused strategy
// removes.  The centroid update merges its per-CTA sums in FP64 scratch and
// the divide step (MatrixBinaryOp::row) reads them from there.
//
// Not carried over: the reference's BufferMap that mirrors buffers across
// OpenCL contexts of different devices (kmeans_three_stage.hpp:337-782).
// All stages run on the one GPU; stages on different queues are ordered with
// events instead of host map/unmap copies.
#pragma once

#include "abstract_kmeans.hpp"
#include "factories.hpp"
#include "timer.hpp"

namespace Clustering {

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class KmeansThreeStage : public AbstractKmeans<PointT, LabelT, MassT, ColMajor> {
public:
    using LabelingFunction = typename LabelingFactory<PointT, LabelT, ColMajor>::LabelingFunction;
    using MassUpdateFunction = typename MassUpdateFactory<LabelT, MassT>::MassUpdateFunction;
    using CentroidUpdateFunction = typename CentroidUpdateFactory<PointT, LabelT, MassT, ColMajor>::CentroidUpdateFunction;

    void run() override {
        if (!q_labeling.valid()) q_labeling = Stream::create();
        if (!q_mass_update.valid()) q_mass_update = q_labeling;
        if (!q_centroid_update.valid()) q_centroid_update = q_mass_update;
        const size_t d = this->num_features, n = this->num_points, k = this->num_clusters;

        points_.resize(n * d);
        centroids_.resize(k * d);
        labels_.resize(n);
        masses_.resize(k);
        {
            auto& dp = this->measurement->add_datapoint().set_name("PointsH2D");
            Event& ev = dp.add_event(q_labeling);
            points_.upload_async(this->in_points(), n * d, q_labeling);
            ev.record_end(q_labeling);
        }
        {
            auto& dp = this->measurement->add_datapoint().set_name("CentroidsH2D");
            Event& ev = dp.add_event(q_labeling);
            centroids_.upload_async(this->io_centroids(), k * d, q_labeling);
            ev.record_end(q_labeling);
        }
        labels_.fill_zero_async(q_labeling);
        masses_.fill_zero_async(q_labeling);
        cu_engine_.reserve((uint32_t)d, (uint32_t)k, q_labeling);
        if (this->centroids_initializer) this->centroids_initializer(points_, centroids_);
        q_labeling.finish();
        this->measurement->set_origin(q_labeling);

        Timer::Timer total_timer;
        total_timer.start();
        Event cu_done;
        this->reset_progress();
        if (this->converge) prev_.resize(k * d);
        // spatial order (as in the single-stage strategy): labeling and
        // centroid update run on a Z-ordered copy, the labeling box-pruned;
        // the last iteration of a full run uses the caller's order
        const bool spatial =
            spatial_order_eligible<PointT, LabelT, MassT, ColMajor>(spatial_mode_, d, n, k, this->max_iterations);
        if (spatial) {
            auto& dp = this->measurement->add_datapoint().set_name("SpatialSort");
            Event& ev = dp.add_event(q_labeling);
            sorted_points_.resize(n * d);
            // the permutation is only needed to bring the labels back when
            // the run can stop early (the last iteration of a full run labels
            // the caller's order directly)
            if (this->converge) perm_.resize(n);
            sort_ws_.resize(ckm_spatial_sort_workspace_bytes(n, (uint32_t)d));
            ckm_check(ckm_spatial_sort_f32((uint32_t)d, n, reinterpret_cast<const float*>(points_.data()),
                                           reinterpret_cast<float*>(sorted_points_.data()),
                                           this->converge ? perm_.data() : nullptr,
                                           sort_ws_.data(), sort_ws_.size(), q_labeling.get()),
                      "SpatialSort");
            ev.record_end(q_labeling);
            cu_done = ev;
        }
        bool labels_sorted = false;
        for (uint32_t it = 0; it < this->max_iterations; ++it) {
            WaitList ll_wait;
            ll_wait.insert(cu_done);
            const bool sorted_it = spatial && it + 1 < this->max_iterations;
            labels_sorted = sorted_it;
            const PointT* it_points = sorted_it ? sorted_points_.data() : points_.data();
            Event ll;
            if (sorted_it) {
                ll_wait.enqueue_wait(q_labeling);
                auto& dp = this->measurement->add_datapoint((int)it).set_name("LabelingSorted");
                Event& ev = dp.add_event(q_labeling);
                ckm_check(ckm_labeling_sorted_f32((uint32_t)d, n, (uint32_t)k,
                                                  reinterpret_cast<const float*>(it_points),
                                                  reinterpret_cast<const float*>(centroids_.data()),
                                                  reinterpret_cast<uint32_t*>(labels_.data()), q_labeling.get()),
                          "LabelingSorted");
                ev.record_end(q_labeling);
                ll = ev;
            } else {
                ll = f_labeling(q_labeling, d, n, k, points_.begin(), points_.end(), centroids_.begin(),
                                centroids_.end(), labels_.begin(), labels_.end(),
                                this->measurement->add_datapoint((int)it), ll_wait);
            }
            WaitList after_ll{ll};
            after_ll.enqueue_wait(q_mass_update);
            masses_.fill_zero_async(q_mass_update);
            Event mu = f_mass_update(q_mass_update, n, k, labels_.begin(), labels_.end(), masses_.begin(),
                                     masses_.end(), this->measurement->add_datapoint((int)it), after_ll);
            WaitList cu_wait{ll, mu};
            // Sums go to FP64 scratch (DEFER); the divide reads them there.
            Event cu = cu_engine_.launch(q_centroid_update, d, n, k, it_points, centroids_.data(),
                                         labels_.data(), masses_.data(), CKM_MODE_DEFER,
                                         this->measurement->add_datapoint((int)it), cu_wait);
            if (this->converge)  // the divide below overwrites the centroids in place
                cuda_check(cudaMemcpyAsync(prev_.data(), centroids_.data(), k * d * sizeof(PointT),
                                           cudaMemcpyDeviceToDevice, q_centroid_update.get()),
                           "centroids copy");
            auto& dv = this->measurement->add_datapoint((int)it).set_name("MatrixBinaryOpRow");
            Event& dev = dv.add_event(q_centroid_update);
            ckm_check(Api<PointT, LabelT, MassT>::finalize((uint32_t)d, (uint32_t)k, centroids_.data(),
                                                          masses_.data(), cu_engine_.scratch().data(),
                                                          cu_engine_.scratch().bytes(), q_centroid_update.get()),
                      "MatrixBinaryOpRow");
            dev.record_end(q_centroid_update);
            cu_done = dev;
            (void)cu;
            if (this->after_iteration(it, probe_, (uint32_t)d, (uint32_t)k, prev_.data(), centroids_.data(),
                                      q_centroid_update))
                break;
        }
        if (labels_sorted) {
            // stopped early on the convergence test: labels back to the
            // caller's order
            q_labeling.finish();
            q_mass_update.finish();
            q_centroid_update.finish();
            labels_out_.resize(n);
            ckm_check(ckm_unpermute_u32(n, perm_.data(), reinterpret_cast<const uint32_t*>(labels_.data()),
                                        reinterpret_cast<uint32_t*>(labels_out_.data()), q_centroid_update.get()),
                      "UnpermuteLabels");
        }
        q_labeling.finish();
        q_mass_update.finish();
        q_centroid_update.finish();
        uint64_t total_time = total_timer.stop<std::chrono::nanoseconds>();
        this->measurement->add_datapoint().set_name("TotalTime").add_value() = total_time;
        last_total_ns_ = total_time;

        download("CentroidsD2H", centroids_, this->io_centroids(), k * d);
        download("LabelsD2H", labels_sorted ? labels_out_ : labels_, this->out_labels(), n);
        download("MassesD2H", masses_, this->out_masses(), k);
        q_centroid_update.finish();
        h2d_bytes_ = (n * d + k * d) * sizeof(PointT);
        d2h_bytes_ = k * d * sizeof(PointT) + n * sizeof(LabelT) + k * sizeof(MassT);
    }

    void set_labeler(LabelingConfiguration config) {
        LabelingFactory<PointT, LabelT, ColMajor> f;
        f_labeling = f.create(config, *this->measurement);
    }
    void set_mass_updater(MassUpdateConfiguration config) {
        MassUpdateFactory<LabelT, MassT> f;
        f_mass_update = f.create(config, *this->measurement);
    }
    void set_centroid_updater(CentroidUpdateConfiguration config) {
        CentroidUpdateFactory<PointT, LabelT, MassT, ColMajor> f;
        cu_engine_ = f.create_engine(config, *this->measurement);
        f_centroid_update = cu_engine_;
    }
    void set_labeling_queue(Stream q) { q_labeling = q; record_device("Labeling", q); }
    void set_mass_update_queue(Stream q) { q_mass_update = q; record_device("MassUpdate", q); }
    void set_centroid_update_queue(Stream q) { q_centroid_update = q; record_device("CentroidUpdate", q); }

    // Spatial order of the iterations (see spatial_order_eligible).
    void set_spatial_order(int mode) { spatial_mode_ = mode; }

    uint64_t last_total_ns() const { return last_total_ns_; }
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }

    LabelingFunction f_labeling;
    MassUpdateFunction f_mass_update;
    CentroidUpdateFunction f_centroid_update;

private:
    void record_device(const std::string& stage, const Stream& q) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, q.device()) == cudaSuccess) {
            this->measurement->set_parameter(stage + "Platform", "CUDA");
            this->measurement->set_parameter(stage + "Device", p.name);
        }
    }
    template <typename T>
    void download(const char* name, const DeviceVector<T>& src, T* dst, size_t count) {
        auto& dp = this->measurement->add_datapoint().set_name(name);
        Event& ev = dp.add_event(q_centroid_update);
        src.download_async(dst, count, q_centroid_update);
        ev.record_end(q_centroid_update);
    }

    CentroidUpdate<PointT, LabelT, MassT> cu_engine_;
    Stream q_labeling, q_mass_update, q_centroid_update;
    DeviceVector<PointT> points_, centroids_, prev_;
    ConvergenceProbe<PointT, LabelT, MassT> probe_;
    DeviceVector<LabelT> labels_, labels_out_;
    DeviceVector<MassT> masses_;
    DeviceVector<PointT> sorted_points_;
    DeviceVector<uint32_t> perm_;
    DeviceVector<unsigned char> sort_ws_;
    int spatial_mode_ = 0;
    uint64_t last_total_ns_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
};

}  // namespace Clustering
