// Configuration structs and the .conf parser.  Struct names and fields are
// the reference's (benchmark_configuration.hpp, kmeans_configuration.hpp,
// labeling_configuration.hpp, mass_update_configuration.hpp,
// centroid_update_configuration.hpp, fused_configuration.hpp); the parser
// accepts the same INI keys (configuration_parser.cpp:43-111) and adds a
// [kmeans.gb300] section for the GB300 build's own knobs.  Unlike the
// reference, unset fields start at defined defaults instead of garbage.
#pragma once

#include <cstddef>
#include <map>
#include <string>
#include <vector>

namespace Clustering {

struct BenchmarkConfiguration {
    size_t runs = 1;
    bool verify = false;
};

struct KmeansConfiguration {
    size_t clusters = 0;
    std::string pipeline;
    size_t iterations = 0;
    bool converge = false;
    std::string point_type = "float";
    std::string label_type = "uint32";
    std::string mass_type = "uint32";
};

struct LabelingConfiguration {
    size_t platform = 0;
    size_t device = 0;
    std::string strategy = "unroll_vector";
    size_t global_size[3] = {0, 1, 1};
    size_t local_size[3] = {0, 1, 1};
    size_t vector_length = 1;
    size_t unroll_clusters_length = 1;
    size_t unroll_features_length = 1;
};

struct MassUpdateConfiguration {
    size_t platform = 0;
    size_t device = 0;
    std::string strategy = "part_local";
    size_t global_size[3] = {0, 1, 1};
    size_t local_size[3] = {0, 1, 1};
    size_t vector_length = 1;
};

struct CentroidUpdateConfiguration {
    size_t platform = 0;
    size_t device = 0;
    std::string strategy = "feature_sum";
    size_t global_size[3] = {0, 1, 1};
    size_t local_size[3] = {0, 1, 1};
    size_t local_features = 1;
    size_t thread_features = 1;
    size_t vector_length = 1;
};

struct FusedConfiguration {
    size_t platform = 0;
    size_t device = 0;
    std::string strategy = "feature_sum";
    size_t global_size[3] = {0, 1, 1};
    size_t local_size[3] = {0, 1, 1};
    size_t vector_length = 1;
};

// [kmeans.gb300]: knobs with no counterpart in the reference.
struct Gb300Configuration {
    size_t device_budget_mib = 0;  // buffered pipelines: device-memory cap (0 = 90% of free memory)
    size_t chunk_mib = 0;          // buffered pipelines: points MiB per chunk (0 = automatic)
    size_t copy_streams = 2;       // buffered pipelines: host<->device copy streams
    bool graphs = true;            // capture the iteration loop in a CUDA graph where possible
    double tolerance = 1e-4;       // kmeans.converge: stop below this relative centroid shift
    int spatial_order = 0;         // single / three stage: iterate on a spatially ordered copy
                                   // ("auto" = 0, "on" = 1, "off" = -1)
};

class ConfigurationParser {
public:
    // Reads an INI file: "[section]" headers, "key = value" lines, '#' or ';'
    // comments.  Keys are section-qualified ("kmeans.fused.strategy").  A
    // size list ("global_size") takes whitespace/comma separated values or
    // repeated lines.  Unknown keys throw std::invalid_argument, like Boost
    // program_options' parse_config_file on an unregistered option.
    void parse_file(std::string file);
    void parse_string(const std::string& text, const std::string& origin = "<string>");

    BenchmarkConfiguration get_benchmark_configuration() const;
    KmeansConfiguration get_kmeans_configuration() const;
    LabelingConfiguration get_labeling_configuration() const;
    MassUpdateConfiguration get_mass_update_configuration() const;
    CentroidUpdateConfiguration get_centroid_update_configuration() const;
    FusedConfiguration get_fused_configuration() const;
    Gb300Configuration get_gb300_configuration() const;

    bool has(const std::string& key) const { return vm_.count(key) != 0; }
    const std::map<std::string, std::vector<std::string>>& values() const { return vm_; }

private:
    std::map<std::string, std::vector<std::string>> vm_;
};

}  // namespace Clustering
