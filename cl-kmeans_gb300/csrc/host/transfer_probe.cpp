// Host <-> device link probe: the throughput of chunked copies between host
// memory (pinned or pageable) and the GPU, the roofline of the buffered
// pipelines (their points stream over this link every iteration).  The
// reference measures the same quantity with transfer_bench.cpp (buffers of
// growing size pushed through its buffer cache, repeated `repeat` times); this
// probe times `repeat` back-to-back copies of one chunk size with CUDA events
// on one stream, so the figure is the link's, not a scheduler's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../ckm_internal.h"

namespace {

struct ProbeBuffers {
    char* host = nullptr;
    bool pinned = false;
    void* dev = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~ProbeBuffers() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
        if (dev) cudaFree(dev);
        if (host) {
            if (pinned) cudaFreeHost(host);
            else std::free(host);
        }
    }
};

}  // namespace

extern "C" int ckm_transfer_probe(int device, uint64_t chunk_bytes, uint32_t repeat, int pinned, int to_device,
                                  uint32_t trials, double* best_gbs, double* mean_gbs) {
    if (chunk_bytes == 0 || repeat == 0 || trials == 0 || !best_gbs)
        return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "chunk_bytes, repeat and trials must be >= 1; best_gbs non-NULL");
    const uint64_t total = chunk_bytes * repeat;
    if (total / repeat != chunk_bytes) return ckm::fail(CKM_ERR_INVALID_ARGUMENT, "chunk_bytes * repeat overflows");
    if (device >= 0) {
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) return ckm::cuda_fail(e, "cudaSetDevice");
    }
    ProbeBuffers b;
    b.pinned = pinned != 0;
    cudaError_t e = cudaSuccess;
    if (b.pinned) {
        e = cudaMallocHost((void**)&b.host, total);
        if (e != cudaSuccess) return ckm::cuda_fail(e, "cudaMallocHost(probe)");
    } else {
        b.host = static_cast<char*>(std::malloc(total));
        if (!b.host) return ckm::fail(CKM_ERR_ALLOC, "host allocation for the probe failed");
    }
    std::memset(b.host, 1, total);  // the pages exist before the timed copies
    if ((e = cudaMalloc(&b.dev, chunk_bytes)) != cudaSuccess) return ckm::cuda_fail(e, "cudaMalloc(probe)");
    if ((e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking)) != cudaSuccess)
        return ckm::cuda_fail(e, "cudaStreamCreate(probe)");
    if ((e = cudaEventCreate(&b.e0)) != cudaSuccess || (e = cudaEventCreate(&b.e1)) != cudaSuccess)
        return ckm::cuda_fail(e, "cudaEventCreate(probe)");
    double best = 0.0, sum = 0.0;
    for (uint32_t t = 0; t <= trials; ++t) {  // trial 0 warms the path up and is not counted
        if ((e = cudaEventRecord(b.e0, b.stream)) != cudaSuccess) return ckm::cuda_fail(e, "cudaEventRecord");
        for (uint32_t r = 0; r < repeat; ++r) {
            char* h = b.host + (uint64_t)r * chunk_bytes;
            e = to_device ? cudaMemcpyAsync(b.dev, h, chunk_bytes, cudaMemcpyHostToDevice, b.stream)
                          : cudaMemcpyAsync(h, b.dev, chunk_bytes, cudaMemcpyDeviceToHost, b.stream);
            if (e != cudaSuccess) return ckm::cuda_fail(e, "cudaMemcpyAsync(probe)");
        }
        if ((e = cudaEventRecord(b.e1, b.stream)) != cudaSuccess) return ckm::cuda_fail(e, "cudaEventRecord");
        if ((e = cudaEventSynchronize(b.e1)) != cudaSuccess) return ckm::cuda_fail(e, "cudaEventSynchronize");
        float ms = 0.0f;
        if ((e = cudaEventElapsedTime(&ms, b.e0, b.e1)) != cudaSuccess) return ckm::cuda_fail(e, "cudaEventElapsedTime");
        if (t == 0) continue;
        const double gbs = ms > 0.0f ? (double)total / (ms * 1e-3) / 1e9 : 0.0;
        best = std::max(best, gbs);
        sum += gbs;
    }
    *best_gbs = best;
    if (mean_gbs) *mean_gbs = sum / trials;
    return CKM_OK;
}
