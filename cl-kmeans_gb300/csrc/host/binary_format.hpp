// Binary feature-file format (binary_format.hpp/.cpp of the reference;
// writer cluster_generator.cpp:157-196):
//   uint64 num_features, uint64 num_clusters (= 0), uint64 num_points
//   float32 points, column-major (all points of feature 0, then feature 1 ...)
// Little-endian.  The reader always reads float32, also into a double
// matrix (binary_format.cpp:39), and rejects files with ground-truth
// centroids (num_clusters != 0, binary_format.cpp:32).  Sizes are 64-bit, so
// files with more than 2^32 values read and write in bounded blocks.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace Clustering {

struct BinaryHeader {
    uint64_t num_features = 0;
    uint64_t num_clusters = 0;
    uint64_t num_points = 0;
};

class BinaryFormat {
public:
    // Reads the header only.  Throws std::runtime_error on a short file.
    static BinaryHeader read_header(const std::string& file);

    // Reads the whole matrix (column-major) into `out` (resized to n * d).
    // Returns 1 like the reference; throws on I/O or format errors.
    template <typename FP>
    int read(const std::string& file, std::vector<FP>& out, uint64_t& num_points, uint64_t& num_features);

    // Reads points [first, first + count) of every feature into `dst`
    // (column-major count x d, caller-allocated, e.g. pinned memory).
    static void read_points(const std::string& file, uint64_t first, uint64_t count, float* dst);

    // Writes a column-major float matrix.
    static void write(const std::string& file, const float* points, uint64_t num_points, uint64_t num_features);
};

}  // namespace Clustering
