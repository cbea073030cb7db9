#include "binary_format.hpp"

#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace Clustering {

namespace {

struct File {
    FILE* f = nullptr;
    File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {
        if (!f) throw std::runtime_error("cannot open \"" + path + "\"");
    }
    ~File() {
        if (f) std::fclose(f);
    }
};

void read_exact(FILE* f, void* dst, size_t bytes, const std::string& what) {
    if (bytes && std::fread(dst, 1, bytes, f) != bytes) throw std::runtime_error("short read: " + what);
}

void seek(FILE* f, uint64_t off) {
    if (fseeko(f, (off_t)off, SEEK_SET) != 0) throw std::runtime_error("seek failed");
}

}  // namespace

BinaryHeader BinaryFormat::read_header(const std::string& file) {
    File fh(file, "rb");
    BinaryHeader h;
    uint64_t v[3];
    read_exact(fh.f, v, sizeof(v), file + " header");
    h.num_features = v[0];
    h.num_clusters = v[1];
    h.num_points = v[2];
    return h;
}

template <typename FP>
int BinaryFormat::read(const std::string& file, std::vector<FP>& out, uint64_t& num_points, uint64_t& num_features) {
    BinaryHeader h = read_header(file);
    if (h.num_clusters != 0) throw std::runtime_error("importing ground-truth centroids is not supported");
    num_points = h.num_points;
    num_features = h.num_features;
    out.resize(h.num_points * h.num_features);
    File fh(file, "rb");
    seek(fh.f, 24);
    const uint64_t total = h.num_points * h.num_features;
    std::vector<float> block(1 << 20);
    for (uint64_t off = 0; off < total; off += block.size()) {
        const uint64_t cnt = std::min<uint64_t>(block.size(), total - off);
        read_exact(fh.f, block.data(), cnt * sizeof(float), file + " body");
        for (uint64_t i = 0; i < cnt; ++i) out[off + i] = (FP)block[i];
    }
    return 1;
}

template int BinaryFormat::read<float>(const std::string&, std::vector<float>&, uint64_t&, uint64_t&);
template int BinaryFormat::read<double>(const std::string&, std::vector<double>&, uint64_t&, uint64_t&);

void BinaryFormat::read_points(const std::string& file, uint64_t first, uint64_t count, float* dst) {
    BinaryHeader h = read_header(file);
    if (first + count > h.num_points) throw std::runtime_error("point range outside the file");
    File fh(file, "rb");
    for (uint64_t f = 0; f < h.num_features; ++f) {
        seek(fh.f, 24 + (f * h.num_points + first) * sizeof(float));
        read_exact(fh.f, dst + f * count, count * sizeof(float), file + " body");
    }
}

void BinaryFormat::write(const std::string& file, const float* points, uint64_t num_points, uint64_t num_features) {
    File fh(file, "wb");
    const uint64_t hdr[3] = {num_features, 0, num_points};
    if (std::fwrite(hdr, sizeof(hdr), 1, fh.f) != 1) throw std::runtime_error("write failed: " + file);
    const uint64_t total = num_points * num_features;
    const uint64_t step = 1 << 24;
    for (uint64_t off = 0; off < total; off += step) {
        const uint64_t cnt = std::min(step, total - off);
        if (std::fwrite(points + off, sizeof(float), cnt, fh.f) != cnt) throw std::runtime_error("write failed: " + file);
    }
}

}  // namespace Clustering
