// The four strategy factories.  Same class names, functor signatures and
// error behaviour as fused_factory.hpp:27-87, labeling_factory.hpp:26-86,
// mass_update_factory.hpp:27-98 and centroid_update_factory.hpp:28-127:
// create() records the launch parameters in the Measurement and throws
// std::invalid_argument(strategy) for an unknown strategy name.
#pragma once

#include <functional>
#include <stdexcept>
#include <string>

#include "kernels.hpp"

namespace Clustering {

template <typename PointT, typename LabelT, typename MassT, bool ColMajor>
class FusedFactory {
public:
    using FusedFunction = std::function<Event(
        Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
        BufferIterator<PointT> points_begin, BufferIterator<PointT> points_end,
        BufferIterator<PointT> old_centroids_begin, BufferIterator<PointT> old_centroids_end,
        BufferIterator<PointT> new_centroids_begin, BufferIterator<PointT> new_centroids_end,
        BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> labels_end, BufferIterator<MassT> masses_begin,
        BufferIterator<MassT> masses_end, Measurement::DataPoint& datapoint, WaitList const& events)>;

    FusedFunction create(FusedConfiguration config, Measurement::Measurement& measurement) {
        return create_engine(config, measurement);
    }

    // The strategy names create() accepts; others throw (fused_factory.hpp:83-85).
    static bool known(const std::string& strategy) {
        return strategy == "cluster_merge" || strategy == "feature_sum";
    }

    // The functor's object, for strategies that also run whole-iteration launches.
    FusedLloyd<PointT, LabelT, MassT> create_engine(FusedConfiguration config, Measurement::Measurement& measurement) {
        measurement.set_parameter("FusedGlobalSize", std::to_string(config.global_size[0]));
        measurement.set_parameter("FusedLocalSize", std::to_string(config.local_size[0]));
        measurement.set_parameter("FusedVectorLength", std::to_string(config.vector_length));
        if (known(config.strategy)) {
            FusedLloyd<PointT, LabelT, MassT> strategy;
            strategy.prepare(config);
            return strategy;
        }
        throw std::invalid_argument(config.strategy);
    }
};

template <typename PointT, typename LabelT, bool ColMajor>
class LabelingFactory {
public:
    using LabelingFunction = std::function<Event(
        Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
        BufferIterator<PointT> points_begin, BufferIterator<PointT> points_end,
        BufferIterator<PointT> centroids_begin, BufferIterator<PointT> centroids_end,
        BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> labels_end, Measurement::DataPoint& datapoint,
        WaitList const& events)>;

    // The strategy names create() accepts; others throw (labeling_factory.hpp:82-84).
    static bool known(const std::string& strategy) { return strategy == "unroll_vector"; }

    LabelingFunction create(LabelingConfiguration config, Measurement::Measurement& measurement) {
        measurement.set_parameter("LabelingGlobalSize", std::to_string(config.global_size[0]));
        measurement.set_parameter("LabelingLocalSize", std::to_string(config.local_size[0]));
        if (known(config.strategy)) {
            measurement.set_parameter("LabelingVectorLength", std::to_string(config.vector_length));
            measurement.set_parameter("LabelingUnrollClustersLength", std::to_string(config.unroll_clusters_length));
            measurement.set_parameter("LabelingUnrollFeaturesLength", std::to_string(config.unroll_features_length));
            LabelingUnrollVector<PointT, LabelT> strategy;
            strategy.prepare(config);
            return strategy;
        }
        throw std::invalid_argument(config.strategy);
    }
};

template <typename LabelT, typename MassT>
class MassUpdateFactory {
public:
    using MassUpdateFunction = std::function<Event(
        Stream queue, size_t num_points, size_t num_clusters, BufferIterator<LabelT> labels_begin,
        BufferIterator<LabelT> labels_end, BufferIterator<MassT> masses_begin, BufferIterator<MassT> masses_end,
        Measurement::DataPoint& datapoint, WaitList const& events)>;

    // The strategy names create() accepts; others throw (mass_update_factory.hpp:91-93).
    static bool known(const std::string& strategy) {
        return strategy == "global_atomic" || strategy == "part_global" || strategy == "part_local" ||
               strategy == "part_private";
    }

    MassUpdateFunction create(MassUpdateConfiguration config, Measurement::Measurement& measurement) {
        measurement.set_parameter("MassUpdateGlobalSize", std::to_string(config.global_size[0]));
        measurement.set_parameter("MassUpdateLocalSize", std::to_string(config.local_size[0]));
        if (config.strategy == "part_private")
            measurement.set_parameter("MassUpdateVectorLength", std::to_string(config.vector_length));
        if (known(config.strategy)) {
            MassUpdate<LabelT, MassT> strategy;
            strategy.prepare(config);
            return strategy;
        }
        throw std::invalid_argument(config.strategy);
    }
};

template <typename PointT, typename LabelT, typename MassT, bool ColMajor>
class CentroidUpdateFactory {
public:
    using CentroidUpdateFunction = std::function<Event(
        Stream queue, size_t num_features, size_t num_points, size_t num_clusters,
        BufferIterator<PointT> points_begin, BufferIterator<PointT> points_end,
        BufferIterator<PointT> centroids_begin, BufferIterator<PointT> centroids_end,
        BufferIterator<LabelT> labels_begin, BufferIterator<LabelT> labels_end, BufferIterator<MassT> masses_begin,
        BufferIterator<MassT> masses_end, Measurement::DataPoint& datapoint, WaitList const& events)>;

    CentroidUpdateFunction create(CentroidUpdateConfiguration config, Measurement::Measurement& measurement) {
        return create_engine(config, measurement);
    }

    // The strategy names create() accepts; others throw (centroid_update_factory.hpp:121-123).
    static bool known(const std::string& strategy) {
        return strategy == "feature_sum" || strategy == "feature_sum_pardim" || strategy == "cluster_merge";
    }

    CentroidUpdate<PointT, LabelT, MassT> create_engine(CentroidUpdateConfiguration config,
                                                        Measurement::Measurement& measurement) {
        measurement.set_parameter("CentroidUpdateGlobalSize", std::to_string(config.global_size[0]));
        measurement.set_parameter("CentroidUpdateLocalSize", std::to_string(config.local_size[0]));
        if (config.strategy == "cluster_merge" || config.strategy == "feature_sum_pardim")
            measurement.set_parameter("CentroidUpdateVectorLength", std::to_string(config.vector_length));
        if (config.strategy == "feature_sum") {
            CentroidUpdate<PointT, LabelT, MassT> s;
            s.prepare(config);
            return s;
        } else if (config.strategy == "feature_sum_pardim") {
            measurement.set_parameter("CentroidUpdateLocalFeatures", std::to_string(config.local_features));
            measurement.set_parameter("CentroidUpdateThreadFeatures", std::to_string(config.thread_features));
            CentroidUpdate<PointT, LabelT, MassT> s;
            s.prepare(config);
            return s;
        } else if (config.strategy == "cluster_merge") {
            CentroidUpdate<PointT, LabelT, MassT> s;
            s.prepare(config);
            return s;
        }
        throw std::invalid_argument(config.strategy);
    }
};

}  // namespace Clustering
