// .conf parser (keys of configuration_parser.cpp:43-111).
#include "configuration.hpp"

#include <algorithm>
#include <cctype>
#include <fstream>
#include <set>
#include <sstream>
#include <stdexcept>

namespace Clustering {

namespace {

enum class Kind { Size, Bool, String, SizeList };

const std::map<std::string, Kind>& known_keys() {
    static const std::map<std::string, Kind> keys = [] {
        std::map<std::string, Kind> m;
        m["benchmark.runs"] = Kind::Size;
        m["benchmark.verify"] = Kind::Bool;
        m["kmeans.clusters"] = Kind::Size;
        m["kmeans.pipeline"] = Kind::String;
        m["kmeans.iterations"] = Kind::Size;
        m["kmeans.converge"] = Kind::Bool;
        m["kmeans.types.point"] = Kind::String;
        m["kmeans.types.label"] = Kind::String;
        m["kmeans.types.mass"] = Kind::String;
        for (const char* stage : {"labeling", "mass_update", "centroid_update", "fused"}) {
            std::string p = std::string("kmeans.") + stage + ".";
            m[p + "platform"] = Kind::Size;
            m[p + "device"] = Kind::Size;
            m[p + "strategy"] = Kind::String;
            m[p + "global_size"] = Kind::SizeList;
            m[p + "local_size"] = Kind::SizeList;
            m[p + "vector_length"] = Kind::Size;
        }
        m["kmeans.labeling.unroll_clusters_length"] = Kind::Size;
        m["kmeans.labeling.unroll_features_length"] = Kind::Size;
        m["kmeans.centroid_update.local_features"] = Kind::Size;
        m["kmeans.centroid_update.thread_features"] = Kind::Size;
        m["kmeans.gb300.device_budget_mib"] = Kind::Size;
        m["kmeans.gb300.chunk_mib"] = Kind::Size;
        m["kmeans.gb300.copy_streams"] = Kind::Size;
        m["kmeans.gb300.graphs"] = Kind::Bool;
        m["kmeans.gb300.tolerance"] = Kind::String;  // a positive real, checked by to_real
        m["kmeans.gb300.spatial_order"] = Kind::String;  // auto | on | off
        return m;
    }();
    return keys;
}

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}

size_t to_size(const std::string& key, const std::string& v) {
    std::string t = trim(v);
    if (t.empty() || t[0] == '-') throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
    size_t pos = 0;
    unsigned long long r = 0;
    try {
        r = std::stoull(t, &pos, 10);
    } catch (...) {
        throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
    }
    if (pos != t.size()) throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
    return (size_t)r;
}

double to_real(const std::string& key, const std::string& v) {
    std::string t = trim(v);
    size_t pos = 0;
    double r = 0.0;
    try {
        r = std::stod(t, &pos);
    } catch (...) {
        throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
    }
    if (pos != t.size() || !(r > 0.0)) throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
    return r;
}

// Boost program_options accepts true/false, yes/no, on/off, 1/0.
bool to_bool(const std::string& key, const std::string& v) {
    std::string t = trim(v);
    std::transform(t.begin(), t.end(), t.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    if (t == "true" || t == "yes" || t == "on" || t == "1") return true;
    if (t == "false" || t == "no" || t == "off" || t == "0") return false;
    throw std::invalid_argument("invalid value for " + key + ": '" + v + "'");
}

std::vector<size_t> to_list(const std::string& key, const std::vector<std::string>& vals) {
    std::vector<size_t> out;
    for (const std::string& v : vals) {
        std::string t = v;
        std::replace(t.begin(), t.end(), ',', ' ');
        std::istringstream is(t);
        std::string tok;
        while (is >> tok) out.push_back(to_size(key, tok));
    }
    return out;
}

// Pads a 1-3 element list with 1 (configuration_parser.cpp:174-191).
void fill3(size_t dst[3], const std::string& key, const std::vector<std::string>& vals) {
    std::vector<size_t> v = to_list(key, vals);
    if (v.empty()) throw std::invalid_argument("empty value for " + key);
    if (v.size() > 3) throw std::invalid_argument("more than 3 values for " + key);
    dst[0] = v[0];
    dst[1] = v.size() > 1 ? v[1] : 1;
    dst[2] = v.size() == 3 ? v[2] : 1;
}

}  // namespace

void ConfigurationParser::parse_file(std::string file) {
    std::ifstream h(file);
    if (!h.is_open()) throw std::invalid_argument("Could not open file \"" + file + "\"");
    std::stringstream ss;
    ss << h.rdbuf();
    parse_string(ss.str(), file);
}

void ConfigurationParser::parse_string(const std::string& text, const std::string& origin) {
    const auto& keys = known_keys();
    std::istringstream is(text);
    std::string line, section;
    size_t lineno = 0;
    std::set<std::string> seen_scalar;
    while (std::getline(is, line)) {
        ++lineno;
        size_t hash = line.find_first_of("#;");
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty()) continue;
        if (line.front() == '[') {
            if (line.back() != ']') throw std::invalid_argument(origin + ":" + std::to_string(lineno) + ": bad section");
            section = trim(line.substr(1, line.size() - 2));
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos)
            throw std::invalid_argument(origin + ":" + std::to_string(lineno) + ": expected key = value");
        std::string key = trim(line.substr(0, eq));
        std::string val = trim(line.substr(eq + 1));
        std::string full = section.empty() ? key : section + "." + key;
        auto it = keys.find(full);
        if (it == keys.end()) throw std::invalid_argument("unrecognised option '" + full + "'");
        if (it->second == Kind::SizeList) {
            vm_[full].push_back(val);
        } else {
            if (seen_scalar.count(full))
                throw std::invalid_argument("option '" + full + "' cannot be specified more than once");
            seen_scalar.insert(full);
            vm_[full] = {val};
        }
    }
}

BenchmarkConfiguration ConfigurationParser::get_benchmark_configuration() const {
    BenchmarkConfiguration c;
    for (auto const& o : vm_) {
        if (o.first == "benchmark.runs") c.runs = to_size(o.first, o.second.back());
        else if (o.first == "benchmark.verify") c.verify = to_bool(o.first, o.second.back());
    }
    return c;
}

KmeansConfiguration ConfigurationParser::get_kmeans_configuration() const {
    KmeansConfiguration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        if (o.first == "kmeans.clusters") c.clusters = to_size(o.first, v);
        else if (o.first == "kmeans.pipeline") c.pipeline = v;
        else if (o.first == "kmeans.iterations") c.iterations = to_size(o.first, v);
        else if (o.first == "kmeans.converge") c.converge = to_bool(o.first, v);
        else if (o.first == "kmeans.types.point") c.point_type = v;
        else if (o.first == "kmeans.types.label") c.label_type = v;
        else if (o.first == "kmeans.types.mass") c.mass_type = v;
    }
    return c;
}

#define CKM_STAGE_COMMON(prefix)                                                   \
    if (o.first == prefix "platform") c.platform = to_size(o.first, v);             \
    else if (o.first == prefix "device") c.device = to_size(o.first, v);            \
    else if (o.first == prefix "strategy") c.strategy = v;                          \
    else if (o.first == prefix "global_size") fill3(c.global_size, o.first, o.second); \
    else if (o.first == prefix "local_size") fill3(c.local_size, o.first, o.second);   \
    else if (o.first == prefix "vector_length") c.vector_length = to_size(o.first, v)

LabelingConfiguration ConfigurationParser::get_labeling_configuration() const {
    LabelingConfiguration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        CKM_STAGE_COMMON("kmeans.labeling.");
        else if (o.first == "kmeans.labeling.unroll_clusters_length") c.unroll_clusters_length = to_size(o.first, v);
        else if (o.first == "kmeans.labeling.unroll_features_length") c.unroll_features_length = to_size(o.first, v);
    }
    return c;
}

MassUpdateConfiguration ConfigurationParser::get_mass_update_configuration() const {
    MassUpdateConfiguration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        CKM_STAGE_COMMON("kmeans.mass_update.");
    }
    return c;
}

CentroidUpdateConfiguration ConfigurationParser::get_centroid_update_configuration() const {
    CentroidUpdateConfiguration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        CKM_STAGE_COMMON("kmeans.centroid_update.");
        else if (o.first == "kmeans.centroid_update.local_features") c.local_features = to_size(o.first, v);
        else if (o.first == "kmeans.centroid_update.thread_features") c.thread_features = to_size(o.first, v);
    }
    return c;
}

FusedConfiguration ConfigurationParser::get_fused_configuration() const {
    FusedConfiguration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        CKM_STAGE_COMMON("kmeans.fused.");
    }
    return c;
}

#undef CKM_STAGE_COMMON

Gb300Configuration ConfigurationParser::get_gb300_configuration() const {
    Gb300Configuration c;
    for (auto const& o : vm_) {
        const std::string& v = o.second.back();
        if (o.first == "kmeans.gb300.device_budget_mib") c.device_budget_mib = to_size(o.first, v);
        else if (o.first == "kmeans.gb300.chunk_mib") c.chunk_mib = to_size(o.first, v);
        else if (o.first == "kmeans.gb300.copy_streams") c.copy_streams = to_size(o.first, v);
        else if (o.first == "kmeans.gb300.graphs") c.graphs = to_bool(o.first, v);
        else if (o.first == "kmeans.gb300.tolerance") c.tolerance = to_real(o.first, v);
        else if (o.first == "kmeans.gb300.spatial_order") {
            if (v == "auto") c.spatial_order = 0;
            else if (v == "on") c.spatial_order = 1;
            else if (v == "off") c.spatial_order = -1;
            else throw std::invalid_argument("kmeans.gb300.spatial_order must be auto, on or off, not '" + v + "'");
        }
    }
    return c;
}

}  // namespace Clustering
