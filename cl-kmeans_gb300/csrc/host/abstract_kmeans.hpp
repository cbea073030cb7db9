// Strategy base class.  Same template, members, setters, getters and
// operator() contract as the reference's AbstractKmeans
// (abstract_kmeans.hpp:24-144): operator() takes host vectors, infers
// k = centroids->size() / num_features, calls run(), and returns (and resets)
// the Measurement.  Device containers are DeviceVector instead of
// boost::compute::vector.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

#include "device.hpp"
#include "measurement.hpp"

namespace Clustering {

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class AbstractKmeans {
public:
    using MeasurementPtr = std::shared_ptr<Measurement::Measurement>;
    template <typename T>
    using Vector = DeviceVector<T>;
    template <typename T>
    using VectorPtr = std::shared_ptr<Vector<T>>;
    template <typename T>
    using HostVector = std::vector<T>;
    template <typename T>
    using HostVectorPtr = std::shared_ptr<std::vector<T>>;

    using InitCentroidsFunction = std::function<void(Vector<PointT>& points, Vector<PointT>& centroids)>;

    AbstractKmeans()
        : max_iterations(0),
          num_features(0),
          num_points(0),
          num_clusters(0),
          host_points(nullptr),
          host_centroids(nullptr),
          host_masses(nullptr),
          host_labels(nullptr),
          measurement(new Measurement::Measurement) {}

    virtual ~AbstractKmeans() {}

    virtual void set_max_iterations(size_t i) { this->max_iterations = i; }
    // `kmeans.converge`: stop once the relative centroid shift of an
    // iteration (max |new - old| / max |old|) is below the tolerance.
    virtual void set_converge(bool c) { this->converge = c; }
    virtual void set_tolerance(double t) { this->tolerance = t > 0.0 ? t : 1e-4; }
    size_t iterations_done() const { return this->done_iterations; }
    bool did_converge() const { return this->converged; }
    float last_shift() const { return this->shift; }

    virtual void set_points(std::shared_ptr<const std::vector<PointT>> p) {
        this->host_points = p;
        if (this->num_features != 0) this->num_points = p->size() / this->num_features;
    }

    virtual void set_features(size_t f) {
        this->num_features = f;
        this->num_points = this->host_points->size() / f;
    }

    virtual void set_clusters(size_t c) { this->num_clusters = c; }

    virtual void set_initializer(InitCentroidsFunction f) { this->centroids_initializer = f; }

    virtual void set_measurement(std::shared_ptr<Measurement::Measurement> m) { this->measurement = m; }

    virtual HostVector<PointT> const& get_centroids() const { return *this->host_centroids; }
    virtual HostVector<LabelT> const& get_labels() const { return *this->host_labels; }
    virtual HostVector<MassT> const& get_cluster_masses() const { return *this->host_masses; }
    virtual Measurement::Measurement const& get_measurement() const { return *this->measurement; }

    virtual void run() = 0;

    virtual MeasurementPtr operator()(size_t max_iterations, size_t num_features,
                                      std::shared_ptr<const std::vector<PointT>> points,
                                      HostVectorPtr<PointT> centroids, HostVectorPtr<MassT> masses,
                                      HostVectorPtr<LabelT> labels) {
        this->max_iterations = max_iterations;
        this->num_features = num_features;
        this->num_points = points->size() / num_features;
        this->num_clusters = centroids->size() / num_features;
        this->host_points = points;
        this->host_centroids = centroids;
        this->host_masses = masses;
        this->host_labels = labels;

        this->run();

        auto current = this->measurement;
        this->measurement.reset(new Measurement::Measurement);
        // strategy parameters (recorded once by the factories) carry over to
        // the next run's measurement; the reference loses them after run 0
        for (const auto& p : current->parameters())
            if (p.first != "TimeStamp") this->measurement->set_parameter(p.first, p.second);
        return current;
    }

    // The same call over raw host arrays (used by the C ABI, which cannot
    // hand out std::vector ownership).  Counts follow the arguments.
    void run_raw(size_t max_iterations, size_t num_features, size_t num_points, size_t num_clusters,
                 const PointT* points, PointT* centroids, MassT* masses, LabelT* labels) {
        this->max_iterations = max_iterations;
        this->num_features = num_features;
        this->num_points = num_points;
        this->num_clusters = num_clusters;
        raw_points = points;
        raw_centroids = centroids;
        raw_masses = masses;
        raw_labels = labels;
        this->run();
        raw_points = nullptr;
        raw_centroids = nullptr;
        raw_masses = nullptr;
        raw_labels = nullptr;
    }

    std::shared_ptr<Measurement::Measurement> current_measurement() const { return measurement; }

protected:
    // Host arrays of the current call (from operator() or run_raw).
    const PointT* in_points() const { return raw_points ? raw_points : host_points->data(); }
    PointT* io_centroids() const { return raw_centroids ? raw_centroids : host_centroids->data(); }
    MassT* out_masses() const { return raw_masses ? raw_masses : host_masses->data(); }
    LabelT* out_labels() const { return raw_labels ? raw_labels : host_labels->data(); }

    // The drivers call this after each iteration; it returns true when the
    // loop should stop (a converging run whose shift fell below tolerance).
    template <typename Probe, typename P>
    bool after_iteration(size_t it, Probe& probe, uint32_t d, uint32_t k, const P* old_c, const P* new_c, Stream& q) {
        this->done_iterations = it + 1;
        if (!this->converge) return false;
        this->converged = probe.converged(d, k, old_c, new_c, this->tolerance, q);
        this->shift = probe.last();
        return this->converged;
    }
    void reset_progress() {
        this->done_iterations = 0;
        this->converged = false;
        this->shift = 0.0f;
    }

    size_t max_iterations;
    bool converge = false;
    double tolerance = 1e-4;
    size_t done_iterations = 0;
    bool converged = false;
    float shift = 0.0f;
    size_t num_features;
    size_t num_points;
    size_t num_clusters;
    std::shared_ptr<const std::vector<PointT>> host_points;
    HostVectorPtr<PointT> host_centroids;
    HostVectorPtr<MassT> host_masses;
    HostVectorPtr<LabelT> host_labels;

    InitCentroidsFunction centroids_initializer;
    std::shared_ptr<Measurement::Measurement> measurement;

    const PointT* raw_points = nullptr;
    PointT* raw_centroids = nullptr;
    MassT* raw_masses = nullptr;
    LabelT* raw_labels = nullptr;
};

}  // namespace Clustering
