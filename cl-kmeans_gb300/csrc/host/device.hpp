// CUDA runtime wrappers used by the host-side strategy layer.  They take the
// place of the Boost.Compute types the reference's strategies are written
// against (boost::compute::vector, buffer_iterator, command_queue, event,
// wait_list; e.g. abstract_kmeans.hpp:28-35, fused_factory.hpp:31-53).
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace Clustering {

class CudaError : public std::runtime_error {
public:
    CudaError(cudaError_t e, const std::string& where)
        : std::runtime_error(where + ": " + cudaGetErrorName(e) + ": " + cudaGetErrorString(e)), code(e) {}
    cudaError_t code;
};

inline void cuda_check(cudaError_t e, const char* where) {
    if (e != cudaSuccess) throw CudaError(e, where);
}

// Device buffers of the strategies come from the current device's default
// stream-ordered pool, set once per device to keep freed memory (no release
// threshold): the multi-GiB buffers of one run are reused by the next instead
// of being mapped and unmapped each time (a free of several GiB took tens of
// milliseconds).  ckm_release_cached_memory() returns the cached memory.
inline void* device_alloc(size_t bytes) {
    static std::once_flag once[64];
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev >= 0 && dev < 64)
        std::call_once(once[dev], [dev]() {
            cudaMemPool_t pool = nullptr;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t keep = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
        });
    void* p = nullptr;
    cuda_check(cudaMallocAsync(&p, bytes, 0), "cudaMallocAsync");
    // ready for every stream before the caller uses it
    cuda_check(cudaStreamSynchronize(0), "cudaStreamSynchronize");
    return p;
}

// The buffer may still be in use by work on any stream: the device finishes
// first (as cudaFree would), then the memory goes back to the pool.
inline void device_free(void* p) {
    cudaDeviceSynchronize();
    cudaFreeAsync(p, 0);
}

// A status from the C ABI that is not CKM_OK.
class KernelError : public std::runtime_error {
public:
    KernelError(int status, const std::string& msg) : std::runtime_error(msg), status(status) {}
    int status;
};

inline uint64_t host_now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// In-order work queue = one CUDA stream (boost::compute::command_queue).
class Stream {
public:
    Stream() = default;
    static Stream create(int device = -1) {
        if (device >= 0) cuda_check(cudaSetDevice(device), "cudaSetDevice");
        cudaStream_t s = nullptr;
        cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        Stream q;
        q.state_ = std::shared_ptr<State>(new State{s, device < 0 ? current_device() : device, true},
                                          [](State* st) {
                                              if (st->owned && st->s) cudaStreamDestroy(st->s);
                                              delete st;
                                          });
        return q;
    }
    static Stream wrap(cudaStream_t s) {
        Stream q;
        q.state_ = std::make_shared<State>(State{s, current_device(), false});
        return q;
    }
    cudaStream_t get() const { return state_ ? state_->s : nullptr; }
    int device() const { return state_ ? state_->device : current_device(); }
    bool valid() const { return (bool)state_; }
    void finish() const { cuda_check(cudaStreamSynchronize(get()), "cudaStreamSynchronize"); }
    uint64_t id() const { return (uint64_t)(uintptr_t)get(); }
    bool operator==(const Stream& o) const { return get() == o.get(); }
    static int current_device() {
        int d = 0;
        cudaGetDevice(&d);
        return d;
    }

private:
    struct State {
        cudaStream_t s;
        int device;
        bool owned;
    };
    std::shared_ptr<State> state_;
};

// Profiling marker pair on a stream (boost::compute::event with profiling):
// start/end CUDA events plus the host enqueue time.
class Event {
public:
    Event() = default;
    static Event record_start(const Stream& q) {
        Event e;
        e.st_ = std::make_shared<State>();
        e.st_->queue_id = q.id();
        e.st_->queued_ns = host_now_ns();
        cuda_check(cudaEventCreate(&e.st_->start), "cudaEventCreate");
        cuda_check(cudaEventCreate(&e.st_->end), "cudaEventCreate");
        cuda_check(cudaEventRecord(e.st_->start, q.get()), "cudaEventRecord");
        return e;
    }
    void record_end(const Stream& q) {
        if (st_) cuda_check(cudaEventRecord(st_->end, q.get()), "cudaEventRecord");
    }
    // A marker for dependencies only (wait lists), recorded now.
    static Event marker(const Stream& q) {
        Event e = record_start(q);
        e.record_end(q);
        return e;
    }
    bool valid() const { return (bool)st_; }
    void wait() const {
        if (st_) cuda_check(cudaEventSynchronize(st_->end), "cudaEventSynchronize");
    }
    cudaEvent_t end_event() const { return st_ ? st_->end : nullptr; }
    cudaEvent_t start_event() const { return st_ ? st_->start : nullptr; }
    uint64_t queue_id() const { return st_ ? st_->queue_id : 0; }
    uint64_t queued_ns() const { return st_ ? st_->queued_ns : 0; }
    // Device duration in ns.
    uint64_t duration_ns() const {
        if (!st_) return 0;
        wait();
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, st_->start, st_->end), "cudaEventElapsedTime");
        return (uint64_t)((double)ms * 1e6);
    }
    // Device time of start / end relative to another event, in ns.
    int64_t start_since(cudaEvent_t base) const { return since(base, st_ ? st_->start : nullptr); }
    int64_t end_since(cudaEvent_t base) const { return since(base, st_ ? st_->end : nullptr); }

private:
    static int64_t since(cudaEvent_t base, cudaEvent_t e) {
        if (!base || !e) return 0;
        cuda_check(cudaEventSynchronize(e), "cudaEventSynchronize");
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, base, e) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return (int64_t)((double)ms * 1e6);
    }
    struct State {
        cudaEvent_t start = nullptr, end = nullptr;
        uint64_t queue_id = 0, queued_ns = 0;
        ~State() {
            if (start) cudaEventDestroy(start);
            if (end) cudaEventDestroy(end);
        }
    };
    std::shared_ptr<State> st_;
};

// boost::compute::wait_list: events a command waits for.
class WaitList {
public:
    WaitList() = default;
    WaitList(std::initializer_list<Event> evs) : events_(evs) {}
    void insert(const Event& e) {
        if (e.valid()) events_.push_back(e);
    }
    void clear() { events_.clear(); }
    bool empty() const { return events_.empty(); }
    size_t size() const { return events_.size(); }
    // Makes `q` wait for every event (no host blocking).
    void enqueue_wait(const Stream& q) const {
        for (const Event& e : events_)
            if (e.valid()) cuda_check(cudaStreamWaitEvent(q.get(), e.end_event(), 0), "cudaStreamWaitEvent");
    }

private:
    std::vector<Event> events_;
};

// boost::compute::buffer_iterator<T>: a typed device pointer with iterator
// arithmetic, so the functors keep the reference's begin/end pairs.
template <typename T>
class BufferIterator {
public:
    BufferIterator() = default;
    explicit BufferIterator(T* p) : p_(p) {}
    T* get() const { return p_; }
    BufferIterator operator+(ptrdiff_t o) const { return BufferIterator(p_ + o); }
    BufferIterator operator-(ptrdiff_t o) const { return BufferIterator(p_ - o); }
    ptrdiff_t operator-(const BufferIterator& o) const { return p_ - o.p_; }
    bool operator==(const BufferIterator& o) const { return p_ == o.p_; }
    bool operator!=(const BufferIterator& o) const { return p_ != o.p_; }

private:
    T* p_ = nullptr;
};

// boost::compute::vector<T>: owning device array.
template <typename T>
class DeviceVector {
public:
    DeviceVector() = default;
    explicit DeviceVector(size_t n) { resize(n); }
    DeviceVector(const DeviceVector&) = delete;
    DeviceVector& operator=(const DeviceVector&) = delete;
    DeviceVector(DeviceVector&& o) noexcept : p_(o.p_), n_(o.n_) {
        o.p_ = nullptr;
        o.n_ = 0;
    }
    DeviceVector& operator=(DeviceVector&& o) noexcept {
        if (this != &o) {
            release();
            p_ = o.p_;
            n_ = o.n_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    ~DeviceVector() { release(); }
    void resize(size_t n) {
        if (n == n_) return;
        release();
        if (n) p_ = static_cast<T*>(device_alloc(n * sizeof(T)));
        n_ = n;
    }
    size_t size() const { return n_; }
    T* data() const { return p_; }
    BufferIterator<T> begin() const { return BufferIterator<T>(p_); }
    BufferIterator<T> end() const { return BufferIterator<T>(p_ + n_); }
    void fill_zero_async(const Stream& q) {
        if (n_) cuda_check(cudaMemsetAsync(p_, 0, n_ * sizeof(T), q.get()), "cudaMemsetAsync");
    }
    void upload_async(const T* src, size_t n, const Stream& q, size_t offset = 0) {
        if (n) cuda_check(cudaMemcpyAsync(p_ + offset, src, n * sizeof(T), cudaMemcpyHostToDevice, q.get()), "H2D");
    }
    void download_async(T* dst, size_t n, const Stream& q, size_t offset = 0) const {
        if (n) cuda_check(cudaMemcpyAsync(dst, p_ + offset, n * sizeof(T), cudaMemcpyDeviceToHost, q.get()), "D2H");
    }
    void swap(DeviceVector& o) noexcept {
        std::swap(p_, o.p_);
        std::swap(n_, o.n_);
    }

private:
    void release() {
        if (p_) device_free(p_);
        p_ = nullptr;
        n_ = 0;
    }
    T* p_ = nullptr;
    size_t n_ = 0;
};

// Page-locked host staging buffer (the reference's CL_MEM_ALLOC_HOST_PTR
// staging slots, simple_buffer_cache.cpp:52-102).
template <typename T>
class PinnedVector {
public:
    PinnedVector() = default;
    explicit PinnedVector(size_t n) { resize(n); }
    PinnedVector(const PinnedVector&) = delete;
    PinnedVector& operator=(const PinnedVector&) = delete;
    PinnedVector(PinnedVector&& o) noexcept : p_(o.p_), n_(o.n_) {
        o.p_ = nullptr;
        o.n_ = 0;
    }
    PinnedVector& operator=(PinnedVector&& o) noexcept {
        if (this != &o) {
            release();
            p_ = o.p_;
            n_ = o.n_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    ~PinnedVector() { release(); }
    void resize(size_t n) {
        if (n == n_) return;
        release();
        if (n) {
            void* p = nullptr;
            cuda_check(cudaHostAlloc(&p, n * sizeof(T), cudaHostAllocDefault), "cudaHostAlloc");
            p_ = static_cast<T*>(p);
        }
        n_ = n;
    }
    T* data() const { return p_; }
    size_t size() const { return n_; }

private:
    void release() {
        if (p_) cudaFreeHost(p_);
        p_ = nullptr;
        n_ = 0;
    }
    T* p_ = nullptr;
    size_t n_ = 0;
};

// Throws KernelError when a C-ABI call did not return CKM_OK.
void ckm_check(int status, const char* where);

}  // namespace Clustering
