// Out-of-core strategies: KmeansSingleStageBuffered
// (kmeans_single_stage_buffered.hpp:37-352) and KmeansThreeStageBuffered
// (kmeans_three_stage_buffered.hpp:37-547), over a chunk streamer that takes
// the place of SimpleBufferCache (simple_buffer_cache.cpp:52-704),
// SingleDeviceScheduler (single_device_scheduler.cpp:108-259) and
// BufferHelper::partition_matrix (buffer_helper.cpp:16-87).
//
// Design:
//   - the points are cut into contiguous point ranges ("chunks"); a chunk of
//     a column-major host matrix is d strided rows, moved with one
//     cudaMemcpy2DAsync, so no host-side re-layout pass is needed;
//   - as many leading chunks as the device budget allows stay resident
//     across iterations (the cache's hits); the rest stream through
//     `slots` device buffers, copy stream -> compute stream -> slot reuse
//     ordered by events (double/triple buffering);
//   - page-locked host memory is copied directly; pageable memory goes
//     through pinned staging slots filled by host worker threads (the
//     reference's IO thread);
//   - per-chunk partial sums accumulate in FP64 scratch (CKM_MODE_DEFER) and
//     one finalize per iteration divides, so chunking does not change the
//     rounding of the centroids;
//   - labels are written back once, after the last iteration (within an
//     iteration they are produced and consumed on the device).
#pragma once

#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <thread>
#include <vector>

#include "abstract_kmeans.hpp"
#include "factories.hpp"
#include "timer.hpp"

namespace Clustering {

class BudgetError : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

struct BufferedOptions {
    uint64_t device_budget_bytes = 0;  // 0: 90% of free device memory
    uint64_t chunk_bytes = 0;          // points bytes per chunk; 0: automatic
    int slots = 3;                     // streaming slots
};

inline bool is_pinned(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Copies rows x bytes with strides using a few host threads.
inline void parallel_copy_2d(char* dst, size_t dpitch, const char* src, size_t spitch, size_t width, size_t rows) {
    const size_t total = width * rows;
    unsigned nt = std::min<unsigned>(8u, std::max(1u, std::thread::hardware_concurrency()));
    if (total < (8u << 20) || nt <= 1) {
        for (size_t r = 0; r < rows; ++r) std::memcpy(dst + r * dpitch, src + r * spitch, width);
        return;
    }
    // split every row into nt pieces
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        th.emplace_back([=] {
            const size_t lo = width * t / nt, hi = width * (t + 1) / nt;
            for (size_t r = 0; r < rows; ++r) std::memcpy(dst + r * dpitch + lo, src + r * spitch + lo, hi - lo);
        });
    }
    for (auto& x : th) x.join();
}

template <typename PointT, typename LabelT>
class ChunkStreamer {
public:
    struct Chunk {
        size_t index, first, count;
        PointT* points;  // device
        LabelT* labels;  // device
        cudaStream_t stream;
    };

    void setup(const PointT* host_points, LabelT* host_labels, size_t n, size_t d, size_t k,
               const BufferedOptions& opt, const Stream& compute) {
        hp_ = host_points;
        hl_ = host_labels;
        n_ = n;
        d_ = d;
        compute_ = compute;
        copy_ = Stream::create(compute.device());
        out_ = Stream::create(compute.device());
        points_pinned_ = n ? is_pinned(host_points) : true;
        labels_pinned_ = n ? is_pinned(host_labels) : true;

        size_t free_b = 0, total_b = 0;
        cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        uint64_t budget = opt.device_budget_bytes ? opt.device_budget_bytes : (uint64_t)(free_b * 0.9);
        if (budget > free_b) throw BudgetError("device budget exceeds free device memory");
        const uint64_t fixed = ckm_scratch_bytes((uint32_t)d, (uint32_t)k) + 4 * k * d * sizeof(PointT) + (1u << 20);
        if (budget <= fixed) throw BudgetError("device budget too small for the centroids and scratch");
        budget -= fixed;
        const size_t per_point = d * sizeof(PointT) + sizeof(LabelT);
        slots_ = std::max(2, opt.slots);
        // points per chunk
        size_t m = opt.chunk_bytes ? opt.chunk_bytes / (d * sizeof(PointT))
                                   : std::min<size_t>(budget / (per_point * (slots_ + 1)), (size_t)(1ull << 31) / (d * sizeof(PointT)));
        m = std::max<size_t>(4, m - m % 4);
        if ((uint64_t)m * per_point * slots_ > budget) throw BudgetError("device budget smaller than the streaming slots");
        chunk_ = std::min(m, std::max<size_t>(n, 4));
        num_chunks_ = n ? (n + chunk_ - 1) / chunk_ : 0;
        // resident chunks: as many as fit beside the streaming slots
        const uint64_t chunk_bytes = (uint64_t)chunk_ * per_point;
        uint64_t left = budget - (uint64_t)chunk_bytes * slots_;
        resident_ = std::min<size_t>(num_chunks_, left / chunk_bytes);
        if (resident_ == num_chunks_) slots_ = 0;  // everything fits: no streaming
        res_points_.resize(resident_);
        res_labels_.resize(resident_);
        for (size_t c = 0; c < resident_; ++c) {
            res_points_[c].resize(chunk_ * d);
            res_labels_[c].resize(chunk_);
        }
        slot_points_.resize(slots_);
        slot_labels_.resize(slots_);
        slot_free_.assign(slots_, Event());
        slot_in_.assign(slots_, Event());
        slot_out_.assign(slots_, Event());
        for (int s = 0; s < slots_; ++s) {
            slot_points_[s].resize(chunk_ * d);
            slot_labels_[s].resize(chunk_);
        }
        if (!points_pinned_ && slots_ + resident_ > 0) {
            stage_.resize(std::max(1, slots_));
            for (auto& b : stage_) b.resize(chunk_ * d);
        }
        loaded_.assign(resident_, false);
        device_bytes_ = (uint64_t)(resident_ + slots_) * chunk_bytes;
    }

    // Runs fn(chunk) for every chunk on the compute stream.  Resident chunks
    // are loaded on first use; the others are streamed through the slots.
    template <typename F>
    void for_each_chunk(F&& fn) {
        for (size_t c = 0; c < num_chunks_; ++c) {
            const size_t first = c * chunk_;
            const size_t count = std::min(chunk_, n_ - first);
            if (c < resident_) {
                if (!loaded_[c]) {
                    upload(res_points_[c].data(), first, count, copy_, 0);
                    Event in = Event::marker(copy_);
                    WaitList{in}.enqueue_wait(compute_);
                    loaded_[c] = true;
                }
                fn(Chunk{c, first, count, res_points_[c].data(), res_labels_[c].data(), compute_.get()});
            } else {
                const int s = (int)((c - resident_) % slots_);
                // the slot's points buffer is free once its previous chunk's
                // compute finished; its labels buffer once they were copied out
                WaitList{slot_free_[s]}.enqueue_wait(copy_);
                upload(slot_points_[s].data(), first, count, copy_, s);
                slot_in_[s] = Event::marker(copy_);
                WaitList{slot_in_[s], slot_out_[s]}.enqueue_wait(compute_);
                fn(Chunk{c, first, count, slot_points_[s].data(), slot_labels_[s].data(), compute_.get()});
                slot_free_[s] = Event::marker(compute_);
                streamed_bytes_ += (uint64_t)count * d_ * sizeof(PointT);
            }
        }
    }

    // Labels of a streamed chunk are copied out right after its compute
    // (call from inside fn on the last iteration).
    void write_back_labels(const Chunk& ch) {
        Event done = Event::marker(compute_);
        WaitList{done}.enqueue_wait(out_);
        if (labels_pinned_) {
            cuda_check(cudaMemcpyAsync(hl_ + ch.first, ch.labels, ch.count * sizeof(LabelT), cudaMemcpyDeviceToHost,
                                       out_.get()),
                       "labels D2H");
        } else {
            // pageable destination: synchronous copy on the out stream
            out_.finish();
            cuda_check(cudaMemcpy(hl_ + ch.first, ch.labels, ch.count * sizeof(LabelT), cudaMemcpyDeviceToHost),
                       "labels D2H");
        }
        d2h_bytes_ += ch.count * sizeof(LabelT);
        // the slot's labels buffer may not be rewritten before they left the device
        if (ch.index >= resident_) slot_out_[(ch.index - resident_) % slots_] = Event::marker(out_);
    }

    // fn(first, count, device labels) for every resident chunk that was loaded.
    template <typename F>
    void for_resident(F&& fn) {
        for (size_t c = 0; c < resident_; ++c)
            if (loaded_[c]) fn(c * chunk_, std::min(chunk_, n_ - c * chunk_), res_labels_[c].data());
    }

    void finish() {
        compute_.finish();
        copy_.finish();
        out_.finish();
    }

    size_t chunk_points() const { return chunk_; }
    size_t num_chunks() const { return num_chunks_; }
    size_t resident_chunks() const { return resident_; }
    int slots() const { return slots_; }
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }
    uint64_t device_bytes() const { return device_bytes_; }

private:
    void upload(PointT* dst, size_t first, size_t count, const Stream& q, int slot) {
        const size_t w = count * sizeof(PointT);
        if (points_pinned_) {
            cuda_check(cudaMemcpy2DAsync(dst, count * sizeof(PointT), hp_ + first, n_ * sizeof(PointT), w, d_,
                                         cudaMemcpyHostToDevice, q.get()),
                       "points H2D");
        } else {
            PinnedVector<PointT>& st = stage_[std::max(0, slot)];
            // the staging slot's previous upload must have left the host
            if (stage_done_.size() < stage_.size()) stage_done_.resize(stage_.size());
            stage_done_[std::max(0, slot)].wait();
            parallel_copy_2d(reinterpret_cast<char*>(st.data()), count * sizeof(PointT),
                             reinterpret_cast<const char*>(hp_ + first), n_ * sizeof(PointT), w, d_);
            cuda_check(cudaMemcpyAsync(dst, st.data(), w * d_, cudaMemcpyHostToDevice, q.get()), "points H2D");
            stage_done_[std::max(0, slot)] = Event::marker(q);
        }
        h2d_bytes_ += (uint64_t)w * d_;
    }

    const PointT* hp_ = nullptr;
    LabelT* hl_ = nullptr;
    size_t n_ = 0, d_ = 0, chunk_ = 0, num_chunks_ = 0, resident_ = 0;
    int slots_ = 0;
    bool points_pinned_ = false, labels_pinned_ = false;
    Stream compute_, copy_, out_;
    std::vector<DeviceVector<PointT>> res_points_, slot_points_;
    std::vector<DeviceVector<LabelT>> res_labels_, slot_labels_;
    std::vector<bool> loaded_;
    std::vector<Event> slot_free_, slot_in_, slot_out_, stage_done_;
    std::vector<PinnedVector<PointT>> stage_;
    uint64_t h2d_bytes_ = 0, d2h_bytes_ = 0, streamed_bytes_ = 0, device_bytes_ = 0;
};

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class KmeansBufferedBase : public AbstractKmeans<PointT, LabelT, MassT, ColMajor> {
public:
    void set_options(const BufferedOptions& o) { opt_ = o; }
    void set_queue(Stream q) { queue_ = q; }
    uint64_t last_total_ns() const { return last_total_ns_; }
    uint64_t h2d_bytes() const { return h2d_bytes_; }
    uint64_t d2h_bytes() const { return d2h_bytes_; }

protected:
    // Shared driver: `per_chunk(chunk, iteration)` enqueues the chunk's work
    // on the compute stream (sums into `scratch` with CKM_MODE_DEFER);
    // finalize() then turns the scratch into the new centroids.
    template <typename PerChunk>
    void drive(Scratch& scratch, PerChunk&& per_chunk) {
        if (!queue_.valid()) queue_ = Stream::create();
        const size_t d = this->num_features, n = this->num_points, k = this->num_clusters;
        old_c_.resize(k * d);
        new_c_.resize(k * d);
        masses_.resize(k);
        old_c_.upload_async(this->io_centroids(), k * d, queue_);
        masses_.fill_zero_async(queue_);
        scratch.reserve((uint32_t)d, (uint32_t)k, queue_);
        streamer_.setup(this->in_points(), this->out_labels(), n, d, k, opt_, queue_);
        this->measurement->set_parameter("BufferedChunkPoints", std::to_string(streamer_.chunk_points()));
        this->measurement->set_parameter("BufferedChunks", std::to_string(streamer_.num_chunks()));
        this->measurement->set_parameter("BufferedResidentChunks", std::to_string(streamer_.resident_chunks()));
        this->measurement->set_parameter("BufferedSlots", std::to_string(streamer_.slots()));
        queue_.finish();
        this->measurement->set_origin(queue_);

        Timer::Timer total_timer;
        total_timer.start();
        this->reset_progress();
        for (uint32_t it = 0; it < this->max_iterations; ++it) {
            // labels of streamed chunks go back to the host in the last
            // iteration; a converging run may stop after any iteration
            const bool last = it + 1 == this->max_iterations || this->converge;
            masses_.fill_zero_async(queue_);
            auto& dp = this->measurement->add_datapoint((int)it).set_name("ChunkLoop");
            Event& ev = dp.add_event(queue_);
            streamer_.for_each_chunk([&](const typename ChunkStreamer<PointT, LabelT>::Chunk& ch) {
                per_chunk(ch, it);
                if (last && ch.index >= streamer_.resident_chunks()) streamer_.write_back_labels(ch);
            });
            ev.record_end(queue_);
            auto& dv = this->measurement->add_datapoint((int)it).set_name("MatrixBinaryOpRow");
            Event& dev = dv.add_event(queue_);
            ckm_check(Api<PointT, LabelT, MassT>::finalize((uint32_t)d, (uint32_t)k, new_c_.data(), masses_.data(),
                                                          scratch.data(), scratch.bytes(), queue_.get()),
                      "finalize");
            dev.record_end(queue_);
            old_c_.swap(new_c_);
            if (this->after_iteration(it, probe_, (uint32_t)d, (uint32_t)k, new_c_.data(), old_c_.data(), queue_))
                break;
        }
        streamer_.finish();
        uint64_t total_time = total_timer.stop<std::chrono::nanoseconds>();
        this->measurement->add_datapoint().set_name("TotalTime").add_value() = total_time;
        last_total_ns_ = total_time;

        old_c_.download_async(this->io_centroids(), k * d, queue_);
        masses_.download_async(this->out_masses(), k, queue_);
        if (this->max_iterations == 0) {
            // no iteration ran: labels stay as the caller passed them
        } else {
            streamer_.for_resident([&](size_t first, size_t count, const LabelT* dl) {
                cuda_check(cudaMemcpyAsync(this->out_labels() + first, dl, count * sizeof(LabelT),
                                           cudaMemcpyDeviceToHost, queue_.get()),
                           "labels D2H");
            });
        }
        queue_.finish();
        h2d_bytes_ = streamer_.h2d_bytes() + k * d * sizeof(PointT);
        d2h_bytes_ = streamer_.d2h_bytes() + k * d * sizeof(PointT) + k * sizeof(MassT) +
                     std::min(n, streamer_.resident_chunks() * streamer_.chunk_points()) * sizeof(LabelT);
    }

    const PointT* old_centroids() const { return old_c_.data(); }

    BufferedOptions opt_;
    Stream queue_;
    ChunkStreamer<PointT, LabelT> streamer_;
    DeviceVector<PointT> old_c_, new_c_;
    DeviceVector<MassT> masses_;
    ConvergenceProbe<PointT, LabelT, MassT> probe_;
    uint64_t last_total_ns_ = 0, h2d_bytes_ = 0, d2h_bytes_ = 0;
};

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class KmeansSingleStageBuffered : public KmeansBufferedBase<PointT, LabelT, MassT, ColMajor> {
public:
    void set_fused(FusedConfiguration config) {
        FusedFactory<PointT, LabelT, MassT, ColMajor> factory;
        engine_ = factory.create_engine(config, *this->measurement);
    }
    void run() override {
        const size_t d = this->num_features, k = this->num_clusters;
        this->drive(engine_.scratch(), [&](const typename ChunkStreamer<PointT, LabelT>::Chunk& ch, uint32_t it) {
            ckm_check(Api<PointT, LabelT, MassT>::fused((uint32_t)d, ch.count, (uint32_t)k, ch.points,
                                                       this->old_centroids(), nullptr, ch.labels, nullptr,
                                                       engine_.scratch().data(), engine_.scratch().bytes(),
                                                       CKM_MODE_DEFER, ch.stream),
                      "FusedFeatureSum");
            (void)it;
        });
    }

private:
    FusedLloyd<PointT, LabelT, MassT> engine_;
};

template <typename PointT, typename LabelT, typename MassT, bool ColMajor = true>
class KmeansThreeStageBuffered : public KmeansBufferedBase<PointT, LabelT, MassT, ColMajor> {
public:
    void set_labeler(LabelingConfiguration c) { ll_ = c; }
    void set_mass_updater(MassUpdateConfiguration c) {
        MassUpdateFactory<LabelT, MassT> f;
        f.create(c, *this->measurement);  // validates the strategy name
    }
    void set_centroid_updater(CentroidUpdateConfiguration c) {
        CentroidUpdateFactory<PointT, LabelT, MassT, ColMajor> f;
        cu_ = f.create_engine(c, *this->measurement);
    }
    void run() override {
        LabelingFactory<PointT, LabelT, ColMajor> lf;
        lf.create(ll_, *this->measurement);  // validates the strategy name
        const size_t d = this->num_features, k = this->num_clusters;
        this->drive(cu_.scratch(), [&](const typename ChunkStreamer<PointT, LabelT>::Chunk& ch, uint32_t) {
            ckm_check(Api<PointT, LabelT, MassT>::labeling((uint32_t)d, ch.count, (uint32_t)k, ch.points,
                                                          this->old_centroids(), ch.labels, ch.stream),
                      "LabelingUnrollVector");
            ckm_check(Api<PointT, LabelT, MassT>::mass(ch.count, (uint32_t)k, ch.labels, this->masses_.data(),
                                                      ch.stream),
                      "MassUpdate");
            ckm_check(Api<PointT, LabelT, MassT>::centroid((uint32_t)d, ch.count, (uint32_t)k, ch.points, nullptr,
                                                          ch.labels, nullptr, cu_.scratch().data(),
                                                          cu_.scratch().bytes(), CKM_MODE_DEFER, ch.stream),
                      "CentroidUpdate");
        });
    }

private:
    LabelingConfiguration ll_;
    CentroidUpdate<PointT, LabelT, MassT> cu_;
};

}  // namespace Clustering
