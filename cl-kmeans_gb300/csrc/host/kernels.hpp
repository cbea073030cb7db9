// Kernel-wrapper layer: host objects that size scratch, record measurement
// events and launch the CUDA kernels through the C ABI.  Each class stands
// where the reference's cl_kernels/*.hpp wrapper of the same role stands
// (FusedFeatureSum, FusedClusterMerge, LabelingUnrollVector, MassUpdate*,
// CentroidUpdate*, MatrixBinaryOp, ReduceVectorParcol); every one is a
// callable with the reference functor signature.
#pragma once

#include <cstdint>
#include <string>
#include <type_traits>

#include "../../../include/ckm.h"
#include "configuration.hpp"
#include "device.hpp"
#include "measurement.hpp"

namespace Clustering {

// Per-type entry points of the C ABI.
template <typename PointT, typename LabelT, typename MassT>
struct Api;

template <>
struct Api<float, uint32_t, uint32_t> {
    static int fused(uint32_t d, uint64_t n, uint32_t k, const float* p, const float* oc, float* nc, uint32_t* l,
                     uint32_t* m, void* s, size_t sb, int mode, cudaStream_t q) {
        return ckm_fused_f32(d, n, k, p, oc, nc, l, m, s, sb, mode, (ckm_stream_t)q);
    }
    static int labeling(uint32_t d, uint64_t n, uint32_t k, const float* p, const float* c, uint32_t* l,
                        cudaStream_t q) {
        return ckm_labeling_f32(d, n, k, p, c, l, (ckm_stream_t)q);
    }
    static int mass(uint64_t n, uint32_t k, const uint32_t* l, uint32_t* m, cudaStream_t q) {
        return ckm_mass_update_u32(n, k, l, m, (ckm_stream_t)q);
    }
    static int centroid(uint32_t d, uint64_t n, uint32_t k, const float* p, float* c, const uint32_t* l,
                        const uint32_t* m, void* s, size_t sb, int mode, cudaStream_t q) {
        return ckm_centroid_update_f32(d, n, k, p, c, l, m, s, sb, mode, (ckm_stream_t)q);
    }
    static int divide(uint32_t d, uint32_t k, float* c, const uint32_t* m, cudaStream_t q) {
        return ckm_matrix_divide_row_f32(d, k, c, m, (ckm_stream_t)q);
    }
    static int shift(uint32_t d, uint32_t k, const float* o, const float* n, float* out, cudaStream_t q) {
        return ckm_centroid_shift_f32(d, k, o, n, out, (ckm_stream_t)q);
    }
    static int add_points(uint64_t n, float* a, const float* b, cudaStream_t q) {
        return ckm_matrix_add_f32(n, a, b, (ckm_stream_t)q);
    }
    static int add_masses(uint64_t n, uint32_t* a, const uint32_t* b, cudaStream_t q) {
        return ckm_matrix_add_u32(n, a, b, (ckm_stream_t)q);
    }
    static int finalize(uint32_t d, uint32_t k, float* c, uint32_t* m, void* s, size_t sb, cudaStream_t q) {
        return ckm_finalize_f32(d, k, c, m, s, sb, (ckm_stream_t)q);
    }
};

template <>
struct Api<double, uint64_t, uint64_t> {
    static int fused(uint32_t d, uint64_t n, uint32_t k, const double* p, const double* oc, double* nc,
                     uint64_t* l, uint64_t* m, void* s, size_t sb, int mode, cudaStream_t q) {
        return ckm_fused_f64(d, n, k, p, oc, nc, l, m, s, sb, mode, (ckm_stream_t)q);
    }
    static int labeling(uint32_t d, uint64_t n, uint32_t k, const double* p, const double* c, uint64_t* l,
                        cudaStream_t q) {
        return ckm_labeling_f64(d, n, k, p, c, l, (ckm_stream_t)q);
    }
    static int mass(uint64_t n, uint32_t k, const uint64_t* l, uint64_t* m, cudaStream_t q) {
        return ckm_mass_update_u64(n, k, l, m, (ckm_stream_t)q);
    }
    static int centroid(uint32_t d, uint64_t n, uint32_t k, const double* p, double* c, const uint64_t* l,
                        const uint64_t* m, void* s, size_t sb, int mode, cudaStream_t q) {
        return ckm_centroid_update_f64(d, n, k, p, c, l, m, s, sb, mode, (ckm_stream_t)q);
    }
    static int divide(uint32_t d, uint32_t k, double* c, const uint64_t* m, cudaStream_t q) {
        return ckm_matrix_divide_row_f64(d, k, c, m, (ckm_stream_t)q);
    }
    static int shift(uint32_t d, uint32_t k, const double* o, const double* n, float* out, cudaStream_t q) {
        return ckm_centroid_shift_f64(d, k, o, n, out, (ckm_stream_t)q);
    }
    static int add_points(uint64_t n, double* a, const double* b, cudaStream_t q) {
        return ckm_matrix_add_f64(n, a, b, (ckm_stream_t)q);
    }
    static int add_masses(uint64_t n, uint64_t* a, const uint64_t* b, cudaStream_t q) {
        return ckm_matrix_add_u64(n, a, b, (ckm_stream_t)q);
    }
    static int finalize(uint32_t d, uint32_t k, double* c, uint64_t* m, void* s, size_t sb, cudaStream_t q) {
        return ckm_finalize_f64(d, k, c, m, s, sb, (ckm_stream_t)q);
    }
};

// FP64 merge scratch owned by a wrapper (sized on first use or by reserve()).
class Scratch {
public:
    void reserve(uint32_t d, uint32_t k, const Stream& q) {
        size_t need = ckm_scratch_bytes(d, k);
        if (buf_.size() < need) {
            buf_.resize(need);
            ckm_check(ckm_scratch_init(buf_.data(), buf_.size(), (ckm_stream_t)q.get()), "ckm_scratch_init");
        }
    }
    void* data() const { return buf_.data(); }
    size_t bytes() const { return buf_.size(); }

private:
    DeviceVector<unsigned char> buf_;
};

// Whether a run uses the spatially ordered copy of its points (FP32,
// column-major, d <= 8, k <= 32, n < 2^32).  mode: 0 = auto (additionally
// n >= 2^20, >= 8 iterations and enough free device memory), 1 = whenever the
// shape allows, -1 = never.
template <typename PointT, typename LabelT, typename MassT, bool ColMajor>
bool spatial_order_eligible(int mode, size_t d, size_t n, size_t k, uint32_t iterations) {
    if (mode < 0) return false;
    if (!(std::is_same<PointT, float>::value && std::is_same<LabelT, uint32_t>::value &&
          std::is_same<MassT, uint32_t>::value && ColMajor))
        return false;
    if (d < 1 || d > 8 || k > 32 || n == 0 || n > 0xffffffffull) return false;
    if (mode > 0) return true;
    if (n < (1ull << 20) || iterations < 8) return false;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
    const size_t need = n * d * sizeof(PointT) + n * 2 * sizeof(LabelT) + ckm_spatial_sort_workspace_bytes(n, (uint32_t)d);
    return need + (size_t(1) << 30) < free_b;
}

// The single-pass fused functor.  `strategy` is the reference's
// kmeans.fused.strategy ("feature_sum" -> FusedFeatureSum,
// fused_feature_sum.hpp:191-444; "cluster_merge" -> FusedClusterMerge,
// fused_cluster_merge.hpp:193-414).  Both names run the same GB300 kernel;
// the name is kept for the measurement record.
template <typename PointT, typename LabelT, typename MassT>
class FusedLloyd {
public:
    void prepare(const FusedConfiguration& config) {
        config_ = config;
        name_ = config.strategy == "cluster_merge" ? "FusedClusterMerge" : "FusedFeatureSum";
    }
    void reserve(uint32_t d, uint32_t k, const Stream& q) { scratch_->reserve(d, k, q); }

    // Reference contract: += sums into new_centroids and counts into masses.
    Event operator()(Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
                     BufferIterator<PointT> points_begin, BufferIterator<PointT> /*points_end*/,
                     BufferIterator<PointT> old_centroids_begin, BufferIterator<PointT> /*old_centroids_end*/,
                     BufferIterator<PointT> new_centroids_begin, BufferIterator<PointT> /*new_centroids_end*/,
                     BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> /*labels_end*/,
                     BufferIterator<MassT> masses_begin, BufferIterator<MassT> /*masses_end*/,
                     Measurement::DataPoint& datapoint, WaitList const& events) {
        return launch(queue, num_features, num_points, num_clusters, points_begin.get(), old_centroids_begin.get(),
                      new_centroids_begin.get(), labels_begin.get(), masses_begin.get(), CKM_MODE_ACCUMULATE,
                      datapoint, events);
    }

    // Any mode (FINALIZE = one whole Lloyd iteration in one launch).
    Event launch(const Stream& queue, size_t d, size_t n, size_t k, const PointT* points, const PointT* old_c,
                 PointT* new_c, LabelT* labels, MassT* masses, int mode, Measurement::DataPoint& dp,
                 WaitList const& events) {
        events.enqueue_wait(queue);
        scratch_->reserve((uint32_t)d, (uint32_t)k, queue);
        dp.set_name(name_);
        Event& ev = dp.add_event(queue);
        ckm_check(Api<PointT, LabelT, MassT>::fused((uint32_t)d, n, (uint32_t)k, points, old_c, new_c, labels,
                                                   masses, scratch_->data(), scratch_->bytes(), mode, queue.get()),
                  name_.c_str());
        ev.record_end(queue);
        return ev;
    }

    Scratch& scratch() { return *scratch_; }

private:
    FusedConfiguration config_;
    std::string name_ = "FusedFeatureSum";
    std::shared_ptr<Scratch> scratch_ = std::make_shared<Scratch>();
};

// LabelingUnrollVector (cl_kernels/labeling_unroll_vector.hpp:168-272).
template <typename PointT, typename LabelT>
class LabelingUnrollVector {
public:
    void prepare(const LabelingConfiguration& config) { config_ = config; }
    Event operator()(Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
                     BufferIterator<PointT> points_begin, BufferIterator<PointT> /*points_end*/,
                     BufferIterator<PointT> centroids_begin, BufferIterator<PointT> /*centroids_end*/,
                     BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> /*labels_end*/,
                     Measurement::DataPoint& datapoint, WaitList const& events) {
        using MassT = LabelT;
        events.enqueue_wait(queue);
        datapoint.set_name("LabelingUnrollVector");
        Event& ev = datapoint.add_event(queue);
        ckm_check(Api<PointT, LabelT, MassT>::labeling((uint32_t)num_features, num_points, (uint32_t)num_clusters,
                                                      points_begin.get(), centroids_begin.get(),
                                                      labels_begin.get(), queue.get()),
                  "LabelingUnrollVector");
        ev.record_end(queue);
        return ev;
    }

private:
    LabelingConfiguration config_;
};

// The four mass-update strategies (cl_kernels/mass_update_*.hpp).  All run
// the same exact shared-memory histogram; the name is recorded.
template <typename LabelT, typename MassT>
class MassUpdate {
public:
    void prepare(const MassUpdateConfiguration& config) {
        config_ = config;
        if (config.strategy == "global_atomic") name_ = "MassUpdateGlobalAtomic";
        else if (config.strategy == "part_global") name_ = "MassUpdatePartGlobal";
        else if (config.strategy == "part_local") name_ = "MassUpdatePartLocal";
        else name_ = "MassUpdatePartPrivate";
    }
    Event operator()(Stream queue, size_t num_points, size_t num_clusters, BufferIterator<LabelT> labels_begin,
                     BufferIterator<LabelT> /*labels_end*/, BufferIterator<MassT> masses_begin,
                     BufferIterator<MassT> /*masses_end*/, Measurement::DataPoint& datapoint,
                     WaitList const& events) {
        using PointT = typename std::conditional<sizeof(LabelT) == 4, float, double>::type;
        events.enqueue_wait(queue);
        datapoint.set_name(name_);
        Event& ev = datapoint.add_event(queue);
        ckm_check(Api<PointT, LabelT, MassT>::mass(num_points, (uint32_t)num_clusters, labels_begin.get(),
                                                  masses_begin.get(), queue.get()),
                  name_.c_str());
        ev.record_end(queue);
        return ev;
    }

private:
    MassUpdateConfiguration config_;
    std::string name_ = "MassUpdatePartLocal";
};

// The three centroid-update strategies (cl_kernels/centroid_update_*.hpp).
template <typename PointT, typename LabelT, typename MassT>
class CentroidUpdate {
public:
    void prepare(const CentroidUpdateConfiguration& config) {
        config_ = config;
        if (config.strategy == "feature_sum_pardim") name_ = "CentroidUpdateFeatureSumPardim";
        else if (config.strategy == "cluster_merge") name_ = "CentroidUpdateClusterMerge";
        else name_ = "CentroidUpdateFeatureSum";
    }
    void reserve(uint32_t d, uint32_t k, const Stream& q) { scratch_->reserve(d, k, q); }

    // Reference contract: += per-label feature sums into centroids.
    Event operator()(Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
                     BufferIterator<PointT> points_begin, BufferIterator<PointT> /*points_end*/,
                     BufferIterator<PointT> centroids_begin, BufferIterator<PointT> /*centroids_end*/,
                     BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> /*labels_end*/,
                     BufferIterator<MassT> masses_begin, BufferIterator<MassT> /*masses_end*/,
                     Measurement::DataPoint& datapoint, WaitList const& events) {
        return launch(queue, num_features, num_points, num_clusters, points_begin.get(), centroids_begin.get(),
                      labels_begin.get(), masses_begin.get(), CKM_MODE_ACCUMULATE, datapoint, events);
    }

    Event launch(const Stream& queue, size_t d, size_t n, size_t k, const PointT* points, PointT* centroids,
                 const LabelT* labels, const MassT* masses, int mode, Measurement::DataPoint& dp,
                 WaitList const& events) {
        events.enqueue_wait(queue);
        scratch_->reserve((uint32_t)d, (uint32_t)k, queue);
        dp.set_name(name_);
        Event& ev = dp.add_event(queue);
        ckm_check(Api<PointT, LabelT, MassT>::centroid((uint32_t)d, n, (uint32_t)k, points, centroids, labels,
                                                      masses, scratch_->data(), scratch_->bytes(), mode,
                                                      queue.get()),
                  name_.c_str());
        ev.record_end(queue);
        return ev;
    }

    Scratch& scratch() { return *scratch_; }

private:
    CentroidUpdateConfiguration config_;
    std::string name_ = "CentroidUpdateFeatureSum";
    std::shared_ptr<Scratch> scratch_ = std::make_shared<Scratch>();
};

// MatrixBinaryOp<PointT, MassT> (cl_kernels/matrix_binary_op.hpp): row()
// with Divide turns sums into means, matrix() with Add accumulates.
template <typename PointT, typename MassT>
class MatrixBinaryOp {
public:
    enum BinaryOp { Add, Sub, Mul, Divide };
    void prepare(BinaryOp op) { op_ = op; }

    Event row(const Stream& queue, size_t num_features, size_t num_clusters, BufferIterator<PointT> matrix_begin,
              BufferIterator<PointT> /*matrix_end*/, BufferIterator<MassT> vector_begin,
              BufferIterator<MassT> /*vector_end*/, Measurement::DataPoint& datapoint, WaitList const& events) {
        using LabelT = MassT;
        if (op_ != Divide) throw std::invalid_argument("MatrixBinaryOp::row supports Divide");
        events.enqueue_wait(queue);
        datapoint.set_name("MatrixBinaryOpRow");
        Event& ev = datapoint.add_event(queue);
        ckm_check(Api<PointT, LabelT, MassT>::divide((uint32_t)num_features, (uint32_t)num_clusters,
                                                    matrix_begin.get(), vector_begin.get(), queue.get()),
                  "MatrixBinaryOpRow");
        ev.record_end(queue);
        return ev;
    }

    template <typename T>
    Event matrix(const Stream& queue, size_t count, BufferIterator<T> a_begin, BufferIterator<T> b_begin,
                 Measurement::DataPoint& datapoint, WaitList const& events) {
        using LabelT = MassT;
        if (op_ != Add) throw std::invalid_argument("MatrixBinaryOp::matrix supports Add");
        events.enqueue_wait(queue);
        datapoint.set_name("MatrixBinaryOpMatrix");
        Event& ev = datapoint.add_event(queue);
        int st;
        if constexpr (std::is_same<T, PointT>::value)
            st = Api<PointT, LabelT, MassT>::add_points(count, a_begin.get(), b_begin.get(), queue.get());
        else
            st = Api<PointT, LabelT, MassT>::add_masses(count, a_begin.get(), b_begin.get(), queue.get());
        ckm_check(st, "MatrixBinaryOpMatrix");
        ev.record_end(queue);
        return ev;
    }

private:
    BinaryOp op_ = Divide;
};

// The `kmeans.converge` test between iterations: the relative centroid
// shift (ckm_centroid_shift_*) is computed on the device and read back
// through a pinned word, which synchronises the stream once per iteration
// (only in converging runs).
template <typename PointT, typename LabelT, typename MassT>
class ConvergenceProbe {
public:
    ConvergenceProbe() = default;
    ConvergenceProbe(const ConvergenceProbe&) = delete;
    ConvergenceProbe& operator=(const ConvergenceProbe&) = delete;
    ~ConvergenceProbe() {
        if (dev_) cudaFree(dev_);
        if (host_) cudaFreeHost(host_);
    }

    // true when the shift from old_c to new_c is below tolerance
    bool converged(uint32_t d, uint32_t k, const PointT* old_c, const PointT* new_c, double tolerance, Stream& q) {
        if (!dev_) {
            cuda_check(cudaMalloc(&dev_, sizeof(float)), "cudaMalloc(shift)");
            cuda_check(cudaMallocHost(&host_, sizeof(float)), "cudaMallocHost(shift)");
        }
        ckm_check(Api<PointT, LabelT, MassT>::shift(d, k, old_c, new_c, dev_, q.get()), "ckm_centroid_shift");
        cuda_check(cudaMemcpyAsync(host_, dev_, sizeof(float), cudaMemcpyDeviceToHost, q.get()), "shift copy");
        q.finish();
        last_ = *host_;
        return last_ < tolerance;
    }
    float last() const { return last_; }

private:
    float* dev_ = nullptr;
    float* host_ = nullptr;
    float last_ = 0.0f;
};

}  // namespace Clustering
