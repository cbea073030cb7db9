// Serving loop: continuous batching of independent k-means jobs.
//
// Three worker threads per server:
//   - the batched lane admits small jobs into device memory (a stream-ordered
//     pool, within the byte budget), then runs rounds: the batch's job table
//     is replaced by the admitted jobs, `round_iterations` persistent
//     launches advance all of them (each parks itself on the device at its
//     own stopping iteration: shift below the tolerance or the cap), and one
//     status read-back per round finds the finished ones.  The lane runs one
//     round ahead (it reads round R - 1's status while R runs), on a stream of
//     the highest priority.  Arrivals join at the next round.
//   - the retire thread copies finished jobs' results to the caller's arrays
//     on its own stream and returns their memory and status slots, after the
//     last round that lists them is done.
//   - the large-job lane runs jobs with n*k*d >= large_work one at a time, on
//     a stream of the lowest priority: on the tensor cores (ckm_tc_fused_f32)
//     when the device and shape allow and d >= 32, else with ckm_fused_f32;
//     the convergence test after every iteration (ckm_centroid_shift_f32).
// Job state per small job lives for the job's whole life: points, labels,
// the centroid pair, masses, FP64 scratch, and a status/ticket slot in two
// server-wide arrays, so a job keeps its iteration count and centroid parity
// across rounds (ckm_batched.h: batch_set_jobs).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ckm_batched.h"
#include "ckm_internal.h"
#include "ckm_tc.h"

using namespace ckm;

namespace {

using Clock = std::chrono::steady_clock;

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

struct SJob {
    ckm_server_job u;
    Clock::time_point t_submit;
    size_t bytes = 0;      // device bytes charged to the budget
    void* block = nullptr; // one pool allocation for all of the job's buffers
    float* d_points = nullptr;
    float* d_cent[2] = {nullptr, nullptr};
    uint32_t* d_labels = nullptr;
    uint32_t* d_masses = nullptr;
    double* d_sums = nullptr;
    unsigned long long* d_msum = nullptr;
    int slot = -1;
    uint64_t joined = 0;   // the first batched round the job is part of
    uint64_t left = 0;     // the round whose status showed it stopped
};

// Byte layout of a small job's block.
struct SmallLayout {
    size_t points, cent0, cent1, labels, masses, sums, msum, total;
};
SmallLayout small_layout(uint64_t n, uint32_t d, uint32_t k) {
    SmallLayout L;
    size_t off = 0;
    L.points = off;
    off += a256((size_t)n * d * 4);
    L.cent0 = off;
    off += a256((size_t)k * d * 4);
    L.cent1 = off;
    off += a256((size_t)k * d * 4);
    L.labels = off;
    off += a256((size_t)std::max<uint64_t>(n, 1) * 4);
    L.masses = off;
    off += a256((size_t)k * 4);
    L.sums = off;
    off += a256((size_t)k * d * 8);
    L.msum = off;
    off += a256((size_t)k * 8);
    L.total = off;
    return L;
}

constexpr uint32_t SLOTS = 65536;  // admitted small jobs at a time

}  // namespace

struct ckm_server {
    ckm_server_options opt{};
    int device = 0;
    uint64_t budget = 0;
    std::atomic<uint64_t> used{0};
    // queues and results
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SJob*> small_q, large_q;
    std::vector<ckm_server_result> results;
    uint64_t submitted = 0, completed = 0;
    bool stop = false;
    std::thread small_thread, large_thread, retire_thread;
    // device
    cudaMemPool_t pool = nullptr;
    cudaStream_t s_up = nullptr, s_comp = nullptr, s_large = nullptr, s_down = nullptr;
    cudaEvent_t ev_up = nullptr, ev_status[2] = {nullptr, nullptr};
    BatchStatus* d_status = nullptr;   // [SLOTS]
    unsigned int* d_tickets = nullptr; // [SLOTS]
    BatchStatus* h_status[2] = {nullptr, nullptr};  // pinned copies, one per round in flight
    std::vector<int> free_slots;
    ::ckm_batch* batch[2] = {nullptr, nullptr};  // job tables of the two rounds in flight
    cudaEvent_t ev_s0[2] = {nullptr, nullptr}, ev_s1[2] = {nullptr, nullptr};
    ckm_server_stats stats{};  // written by the batched lane under mu
    // finished jobs of the batched lane, handed to the retire thread: their
    // results are copied out after the round's event, then they are released
    struct Retiring {
        cudaEvent_t ev;              // recorded on s_comp after the round
        std::vector<SJob*> jobs;
        std::vector<BatchStatus> status;
    };
    std::mutex rmu;
    std::condition_variable cv_retire;
    std::deque<Retiring> retire_q;
    std::vector<cudaEvent_t> free_events;
    bool retire_stop = false;
    uint64_t retiring_jobs = 0;      // queued or being copied out (under rmu)
};

namespace {

void finish(ckm_server* S, SJob* j, int status, uint32_t its, uint32_t conv, float shift, uint32_t lane) {
    ckm_server_result r;
    r.tag = j->u.tag;
    r.status = status;
    r.iterations = its;
    r.converged = conv;
    r.shift = shift;
    r.lane = lane;
    r.first_round = lane == 0 ? j->joined : 0;
    r.last_round = lane == 0 ? j->left : 0;
    r.latency_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - j->t_submit).count();
    std::memset(r.error, 0, sizeof(r.error));
    if (status != CKM_OK) {  // the lane's thread set the message
        const char* m = ckm_last_error();
        std::strncpy(r.error, (m && *m) ? m : ckm_status_string(status), sizeof(r.error) - 1);
    }
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->results.push_back(r);
        ++S->completed;
    }
    S->cv_done.notify_all();
    delete j;
}

// Charges `bytes` to the budget if they fit; false otherwise.
bool charge(ckm_server* S, uint64_t bytes) {
    uint64_t cur = S->used.load();
    while (cur + bytes <= S->budget)
        if (S->used.compare_exchange_weak(cur, cur + bytes)) return true;
    return false;
}

// ---------------------------------------------------------------------------
// Batched lane
// ---------------------------------------------------------------------------

// A small job's block from the pool; points and initial centroids copied
// in; FP64 scratch, status slot and ticket zeroed (all on s_up).
int admit_small(ckm_server* S, SJob* j) {
    const uint64_t n = j->u.num_points;
    const uint32_t d = j->u.num_features, k = j->u.num_clusters;
    const SmallLayout L = small_layout(n, d, k);
    cudaError_t e = cudaMallocFromPoolAsync(&j->block, L.total, S->pool, S->s_up);
    if (e != cudaSuccess) {
        j->block = nullptr;
        return cuda_fail(e, "server: device allocation");
    }
    char* b = static_cast<char*>(j->block);
    j->d_points = reinterpret_cast<float*>(b + L.points);
    j->d_cent[0] = reinterpret_cast<float*>(b + L.cent0);
    j->d_cent[1] = reinterpret_cast<float*>(b + L.cent1);
    j->d_labels = reinterpret_cast<uint32_t*>(b + L.labels);
    j->d_masses = reinterpret_cast<uint32_t*>(b + L.masses);
    j->d_sums = reinterpret_cast<double*>(b + L.sums);
    j->d_msum = reinterpret_cast<unsigned long long*>(b + L.msum);
    if (n) e = cudaMemcpyAsync(j->d_points, j->u.points, (size_t)n * d * 4, cudaMemcpyHostToDevice, S->s_up);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(j->d_cent[0], j->u.init_centroids, (size_t)k * d * 4, cudaMemcpyHostToDevice, S->s_up);
    if (e == cudaSuccess) e = cudaMemsetAsync(b + L.sums, 0, L.total - L.sums, S->s_up);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->d_status + j->slot, 0, sizeof(BatchStatus), S->s_up);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->d_tickets + j->slot, 0, sizeof(unsigned int), S->s_up);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "server: upload");
}

void release_small(ckm_server* S, SJob* j, cudaStream_t s) {
    if (j->block) cudaFreeAsync(j->block, s);
    j->block = nullptr;
    S->used -= j->bytes;
    std::lock_guard<std::mutex> g(S->mu);
    if (j->slot >= 0) S->free_slots.push_back(j->slot);
    j->slot = -1;
}

// Takes queued jobs that fit the budget and the free slots and issues their
// uploads on s_up; they join the next round.
void take_and_admit(ckm_server* S, std::vector<SJob*>& pending, uint64_t& admit_ns, uint64_t& admitted) {
    std::vector<SJob*> take;
    {
        std::lock_guard<std::mutex> g(S->mu);
        while (!S->small_q.empty() && !S->free_slots.empty()) {
            SJob* j = S->small_q.front();
            if (!charge(S, j->bytes)) break;  // waits until retirements free memory
            S->small_q.pop_front();
            j->slot = S->free_slots.back();
            S->free_slots.pop_back();
            take.push_back(j);
        }
    }
    if (take.empty()) return;
    const auto t0 = Clock::now();
    for (SJob* j : take) {
        const int st = admit_small(S, j);
        if (st) {
            release_small(S, j, S->s_up);
            finish(S, j, st, 0, 0, 0.f, 0);
        } else {
            pending.push_back(j);
        }
    }
    admit_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
    admitted += take.size();
}

// The retire thread: for each batch of finished jobs, waits for the round
// (its event), copies every job's centroids, masses and labels to the
// caller's host arrays (pageable copies block this thread, not the lane),
// then releases the jobs' memory and slots and posts their results.
void retire_loop(ckm_server* S) {
    cudaSetDevice(S->device);
    const float tol = S->opt.tolerance;
    for (;;) {
        ckm_server::Retiring r;
        {
            std::unique_lock<std::mutex> lk(S->rmu);
            S->cv_retire.wait(lk, [&] { return S->retire_stop || !S->retire_q.empty(); });
            if (S->retire_q.empty()) break;  // stop requested and nothing left
            r = std::move(S->retire_q.front());
            S->retire_q.pop_front();
        }
        cudaError_t e = cudaStreamWaitEvent(S->s_down, r.ev, 0);
        for (size_t i = 0; i < r.jobs.size() && e == cudaSuccess; ++i) {
            SJob* j = r.jobs[i];
            const BatchStatus& b = r.status[i];
            const size_t kd = (size_t)j->u.num_clusters * j->u.num_features;
            e = cudaMemcpyAsync(j->u.centroids, j->d_cent[b.parity & 1u], kd * 4, cudaMemcpyDeviceToHost, S->s_down);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(j->u.masses, j->d_masses, (size_t)j->u.num_clusters * 4, cudaMemcpyDeviceToHost,
                                    S->s_down);
            if (e == cudaSuccess && j->u.labels && j->u.num_points)
                e = cudaMemcpyAsync(j->u.labels, j->d_labels, (size_t)j->u.num_points * 4, cudaMemcpyDeviceToHost,
                                    S->s_down);
        }
        const cudaError_t es = cudaStreamSynchronize(S->s_down);
        if (e == cudaSuccess) e = es;
        for (size_t i = 0; i < r.jobs.size(); ++i) {
            SJob* j = r.jobs[i];
            const BatchStatus& b = r.status[i];
            release_small(S, j, S->s_down);
            int st = e == cudaSuccess ? CKM_OK : cuda_fail(e, "server: results");
            if (st == CKM_OK && (b.flags & 4u))
                st = fail(CKM_ERR_TIMEOUT, "server: a wait for the tensor cores timed out in the job's round");
            finish(S, j, st, b.iterations, (tol > 0.f && b.shift < tol) ? 1u : 0u, b.shift, 0);
        }
        {
            std::lock_guard<std::mutex> g(S->rmu);
            S->free_events.push_back(r.ev);
            S->retiring_jobs -= r.jobs.size();
        }
        S->cv_work.notify_all();  // memory and slots are free again
    }
}

uint64_t retiring_count(ckm_server* S) {
    std::lock_guard<std::mutex> g(S->rmu);
    return S->retiring_jobs;
}

// The batched lane.  A round: the admitted jobs become the batch's table,
// `round_iterations` launches advance them, the status comes back.  The lane
// runs one round ahead: it launches round R, then reads the status of round
// R - 1 while R runs, so the device never waits for the host between rounds.
// Round R's table is built before R - 1's results are known, so it still
// lists the jobs that stopped in R - 1; they are parked on the device (status
// flags) and the kernel skips them, and their memory and status slots are
// released only after R is done (the retire thread waits for an event
// recorded behind R's launches).  The two rounds in flight use two batch
// objects, two pinned status copies and two sets of events.  Uploads of the
// next jobs are issued while the rounds run; finished jobs go to the retire
// thread, which copies their results out on its own stream.
void small_lane(ckm_server* S) {
    cudaSetDevice(S->device);
    const float tol = S->opt.tolerance;
    const uint32_t max_it = S->opt.max_iterations, rounds = S->opt.round_iterations;
    std::vector<SJob*> active, pending;
    std::vector<BatchJobDev> dev;
    uint64_t round_id = 0;  // rounds launched so far
    // the round launched last, whose status has not been read yet
    bool in_flight = false;
    int fl_par = 0;
    uint64_t fl_id = 0;
    int par = 0;
    auto fail_all = [&](int st) {
        cudaStreamSynchronize(S->s_comp);
        for (SJob* j : active) {
            release_small(S, j, S->s_comp);
            finish(S, j, st, 0, 0, 0.f, 0);
        }
        active.clear();
        in_flight = false;
    };
    for (;;) {
        uint64_t admit_ns = 0, admitted = 0;
        take_and_admit(S, pending, admit_ns, admitted);
        if (active.empty() && pending.empty() && !in_flight) {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop && S->small_q.empty() && retiring_count(S) == 0) break;
            if (S->small_q.empty())
                S->cv_work.wait_for(lk, std::chrono::milliseconds(10), [&] { return S->stop || !S->small_q.empty(); });
            else  // queued jobs wait for retirements to free memory or slots
                S->cv_work.wait_for(lk, std::chrono::milliseconds(1));
            continue;
        }
        const auto t_round = Clock::now();
        if (!pending.empty()) {
            cudaEventRecord(S->ev_up, S->s_up);
            cudaStreamWaitEvent(S->s_comp, S->ev_up, 0);
            for (SJob* j : pending) j->joined = round_id + 1;
            active.insert(active.end(), pending.begin(), pending.end());
            pending.clear();
        }

        // launch round round_id + 1 over every admitted job
        bool launched = false;
        int st = CKM_OK;
        if (!active.empty()) {
            dev.resize(active.size());
            int max_slot = 0;
            for (size_t i = 0; i < active.size(); ++i) {
                const SJob* j = active[i];
                BatchJobDev& J = dev[i];
                J.points = j->d_points;
                J.cent[0] = j->d_cent[0];
                J.cent[1] = j->d_cent[1];
                J.labels = j->d_labels;
                J.masses = j->d_masses;
                J.sums = j->d_sums;
                J.msum = j->d_msum;
                J.ticket = S->d_tickets + j->slot;
                J.status = S->d_status + j->slot;
                J.n = j->u.num_points;
                J.d = j->u.num_features;
                J.k = j->u.num_clusters;
                J.num_tiles = 0;
                J.pad = 0;
                max_slot = std::max(max_slot, j->slot);
            }
            // one 512-thread CTA per SM with the whole shared memory (room for
            // the tensor-core tiles of d = 32 / 64 jobs), 4096-point tiles
            st = batch_set_jobs(S->batch[par], dev.data(), (uint32_t)dev.size(), 4096, 1, tol, max_it, S->s_comp);
            cudaEventRecord(S->ev_s0[par], S->s_comp);
            for (uint32_t r = 0; r < rounds && st == CKM_OK; ++r) st = batch_launch_step(S->batch[par], S->s_comp);
            cudaEventRecord(S->ev_s1[par], S->s_comp);
            if (st == CKM_OK) {
                cudaError_t e = cudaMemcpyAsync(S->h_status[par], S->d_status,
                                                (size_t)(max_slot + 1) * sizeof(BatchStatus), cudaMemcpyDeviceToHost,
                                                S->s_comp);
                if (e == cudaSuccess) e = cudaEventRecord(S->ev_status[par], S->s_comp);
                if (e != cudaSuccess) st = cuda_fail(e, "server: status read-back");
            }
            launched = st == CKM_OK;
        }
        if (st != CKM_OK) {  // the round failed: its jobs fail with the reason
            fail_all(st);
            continue;
        }
        if (launched) ++round_id;

        // while it runs: the next jobs' uploads, and the round before it
        take_and_admit(S, pending, admit_ns, admitted);
        const size_t njobs = active.size();
        size_t ndone = 0;
        float steps_ms = 0.f;
        const auto t_retire = Clock::now();
        if (in_flight) {
            const cudaError_t e = cudaEventSynchronize(S->ev_status[fl_par]);
            if (e != cudaSuccess) {
                fail_all(cuda_fail(e, "server: status read-back"));
                continue;
            }
            cudaEventElapsedTime(&steps_ms, S->ev_s0[fl_par], S->ev_s1[fl_par]);
            // the jobs of that round that stopped go to the retire thread; the
            // event is recorded behind the round launched above, which still
            // lists them
            std::vector<SJob*> keep;
            ckm_server::Retiring r;
            for (SJob* j : active) {
                const BatchStatus& b = S->h_status[fl_par][j->slot];
                if (j->joined > fl_id || !(b.flags & 2u)) {
                    keep.push_back(j);
                    continue;
                }
                j->left = fl_id;
                r.jobs.push_back(j);
                r.status.push_back(b);
            }
            if (!r.jobs.empty()) {
                cudaEvent_t ev = nullptr;
                {
                    std::lock_guard<std::mutex> g(S->rmu);
                    if (!S->free_events.empty()) {
                        ev = S->free_events.back();
                        S->free_events.pop_back();
                    }
                }
                if (!ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
                r.ev = ev;
                cudaEventRecord(r.ev, S->s_comp);
                {
                    std::lock_guard<std::mutex> g(S->rmu);
                    S->retiring_jobs += r.jobs.size();
                    S->retire_q.push_back(std::move(r));
                }
                S->cv_retire.notify_one();
            }
            ndone = active.size() - keep.size();
            active.swap(keep);
        }
        in_flight = launched;
        if (launched) {
            fl_par = par;
            fl_id = round_id;
            par ^= 1;
        }
        const auto t_end = Clock::now();
        {
            std::lock_guard<std::mutex> g(S->mu);
            ckm_server_stats& x = S->stats;
            x.rounds += launched ? 1 : 0;
            x.job_rounds += launched ? njobs : 0;
            x.busy_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t_end - t_round).count();
            x.steps_gpu_ns += (uint64_t)(steps_ms * 1e6);
            x.admit_ns += admit_ns;
            x.retire_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t_end - t_retire).count();
            x.jobs_admitted += admitted;
            x.jobs_completed += ndone;
        }
    }
}

// ---------------------------------------------------------------------------
// Large-job lane
// ---------------------------------------------------------------------------

bool large_uses_tc(const ckm_server_job& u) {
    return u.num_features >= 32 && u.num_points >= 4096 && ckm_tc_supported(u.num_features, u.num_clusters);
}

// Device bytes of a large job: its arrays, the FP64 scratch and, on the
// tensor-core path, the prepared point set and the workspace.
size_t large_bytes(const ckm_server_job& u) {
    const uint64_t n = u.num_points;
    const uint32_t d = u.num_features, k = u.num_clusters;
    size_t b = a256((size_t)n * d * 4) + 2 * a256((size_t)k * d * 4) + a256((size_t)n * 4) + a256((size_t)k * 4) +
               a256(ckm_scratch_bytes(d, k)) + 256;
    if (large_uses_tc(u)) b += a256(ckm_tc_points_bytes(n, d)) + a256(ckm_tc_workspace_bytes(n, d, k));
    return b;
}

int run_large(ckm_server* S, SJob* j, uint32_t* its_out, uint32_t* conv_out, float* shift_out, float* h_shift) {
    const uint64_t n = j->u.num_points;
    const uint32_t d = j->u.num_features, k = j->u.num_clusters;
    const bool tc = large_uses_tc(j->u);
    cudaStream_t s = S->s_large;
    cudaError_t e = cudaMallocFromPoolAsync(&j->block, j->bytes, S->pool, s);
    if (e != cudaSuccess) {
        j->block = nullptr;
        return cuda_fail(e, "server: device allocation");
    }
    char* b = static_cast<char*>(j->block);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char* p = b + off;
        off += a256(bytes);
        return p;
    };
    float* P = reinterpret_cast<float*>(take((size_t)n * d * 4));
    float* C[2] = {reinterpret_cast<float*>(take((size_t)k * d * 4)), reinterpret_cast<float*>(take((size_t)k * d * 4))};
    uint32_t* lab = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
    uint32_t* mass = reinterpret_cast<uint32_t*>(take((size_t)k * 4));
    const size_t sb = ckm_scratch_bytes(d, k);
    void* scratch = take(sb);
    float* d_shift = reinterpret_cast<float*>(take(4));
    void *tcp = nullptr, *ws = nullptr;
    size_t pb = 0, wb = 0;
    if (tc) {
        pb = ckm_tc_points_bytes(n, d);
        wb = ckm_tc_workspace_bytes(n, d, k);
        tcp = take(pb);
        ws = take(wb);
    }
    int st = CKM_OK;
    e = cudaMemcpyAsync(P, j->u.points, (size_t)n * d * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(C[0], j->u.init_centroids, (size_t)k * d * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = cuda_fail(e, "server: upload");
    if (!st) st = ckm_scratch_init(scratch, sb, (ckm_stream_t)s);
    if (!st && tc) st = ckm_tc_prepare_points(d, n, P, tcp, pb, (ckm_stream_t)s);
    const float tol = S->opt.tolerance;
    uint32_t its = 0, conv = 0, cur = 0;
    float shift = 0.f;
    while (!st && its < S->opt.max_iterations) {
        st = tc ? ckm_tc_fused_f32(d, n, k, P, tcp, C[cur], C[cur ^ 1], lab, mass, scratch, sb, ws, wb,
                                   CKM_MODE_FINALIZE, nullptr, (ckm_stream_t)s)
                : ckm_fused_f32(d, n, k, P, C[cur], C[cur ^ 1], lab, mass, scratch, sb, CKM_MODE_FINALIZE,
                                (ckm_stream_t)s);
        if (!st) st = ckm_centroid_shift_f32(d, k, C[cur], C[cur ^ 1], d_shift, (ckm_stream_t)s);
        if (!st) {
            e = cudaMemcpyAsync(h_shift, d_shift, 4, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) st = cuda_fail(e, "server: shift read-back");
        }
        if (st) break;
        cur ^= 1u;
        ++its;
        shift = *h_shift;
        if (tol > 0.f && shift < tol) {
            conv = 1;
            break;
        }
    }
    if (!st) {
        e = cudaMemcpyAsync(j->u.centroids, C[cur], (size_t)k * d * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(j->u.masses, mass, (size_t)k * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && j->u.labels)
            e = cudaMemcpyAsync(j->u.labels, lab, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_fail(e, "server: results");
    }
    cudaFreeAsync(j->block, s);
    cudaStreamSynchronize(s);
    j->block = nullptr;
    *its_out = its;
    *conv_out = conv;
    *shift_out = shift;
    return st;
}

void large_lane(ckm_server* S) {
    cudaSetDevice(S->device);
    float* h_shift = nullptr;
    cudaMallocHost(&h_shift, sizeof(float));
    for (;;) {
        SJob* j = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->large_q.empty(); });
            if (S->large_q.empty()) break;  // stopping
            j = S->large_q.front();
            S->large_q.pop_front();
        }
        while (!charge(S, j->bytes)) std::this_thread::sleep_for(std::chrono::milliseconds(1));
        uint32_t its = 0, conv = 0;
        float shift = 0.f;
        const int st = h_shift ? run_large(S, j, &its, &conv, &shift, h_shift)
                               : fail(CKM_ERR_ALLOC, "server: pinned host allocation failed");
        S->used -= j->bytes;
        finish(S, j, st, its, conv, shift, large_uses_tc(j->u) ? 1u : 2u);
    }
    if (h_shift) cudaFreeHost(h_shift);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int ckm_server_create(const ckm_server_options* options, ckm_server** out) {
    if (!out) return fail(CKM_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    std::unique_ptr<ckm_server> S(new ckm_server());
    if (options) S->opt = *options;
    if (!(S->opt.tolerance > 0.f)) S->opt.tolerance = 1e-4f;
    if (!S->opt.max_iterations) S->opt.max_iterations = 50;
    if (!S->opt.round_iterations) S->opt.round_iterations = 4;
    if (!S->opt.large_work) S->opt.large_work = 1ull << 33;
    S->device = S->opt.device;
    cudaError_t e = cudaSetDevice(S->device);
    if (e != cudaSuccess) return cuda_fail(e, "server: cudaSetDevice");
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return cuda_fail(e, "server: cudaMemGetInfo");
    S->budget = S->opt.device_budget_bytes ? S->opt.device_budget_bytes : free_b / 2;
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = S->device;
    if ((e = cudaMemPoolCreate(&S->pool, &props)) != cudaSuccess) return cuda_fail(e, "server: cudaMemPoolCreate");
    uint64_t keep = ~0ull;  // memory returned to the pool stays there for the next jobs
    cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    // the batched lane's kernels run at the highest stream priority: when a
    // large job's kernel ends, the next round's launch takes the SMs before
    // the large job's next kernel, so small jobs do not queue behind it
    int prio_low = 0, prio_high = 0;
    if ((e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high)) != cudaSuccess)
        return cuda_fail(e, "server: stream priorities");
    if ((e = cudaStreamCreateWithFlags(&S->s_up, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&S->s_comp, cudaStreamNonBlocking, prio_high)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&S->s_large, cudaStreamNonBlocking, prio_low)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&S->s_down, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&S->ev_up, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&S->ev_status[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&S->ev_status[1], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&S->ev_s0[0])) != cudaSuccess || (e = cudaEventCreate(&S->ev_s1[0])) != cudaSuccess ||
        (e = cudaEventCreate(&S->ev_s0[1])) != cudaSuccess || (e = cudaEventCreate(&S->ev_s1[1])) != cudaSuccess)
        return cuda_fail(e, "server: streams");
    if ((e = cudaMalloc(&S->d_status, SLOTS * sizeof(BatchStatus))) != cudaSuccess ||
        (e = cudaMalloc(&S->d_tickets, SLOTS * sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaMallocHost(&S->h_status[0], SLOTS * sizeof(BatchStatus))) != cudaSuccess ||
        (e = cudaMallocHost(&S->h_status[1], SLOTS * sizeof(BatchStatus))) != cudaSuccess)
        return cuda_fail(e, "server: status slots");
    S->free_slots.resize(SLOTS);
    for (uint32_t i = 0; i < SLOTS; ++i) S->free_slots[i] = (int)(SLOTS - 1 - i);
    int st = batch_create_external(&S->batch[0]);
    if (st == CKM_OK) st = batch_create_external(&S->batch[1]);
    if (st) return st;
    ckm_server* raw = S.release();
    raw->retire_thread = std::thread(retire_loop, raw);
    raw->small_thread = std::thread(small_lane, raw);
    raw->large_thread = std::thread(large_lane, raw);
    *out = raw;
    return CKM_OK;
}

int ckm_server_submit(ckm_server* S, const ckm_server_job* job) {
    if (!S || !job) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL argument");
    const ckm_server_job& u = *job;
    if (u.num_points == 0 || u.num_features == 0 || u.num_clusters == 0)
        return fail(CKM_ERR_INVALID_ARGUMENT, "num_points, num_features and num_clusters must be >= 1");
    if (!u.points || !u.init_centroids || !u.centroids || !u.masses)
        return fail(CKM_ERR_INVALID_ARGUMENT, "points, init_centroids, centroids and masses must be non-NULL");
    if ((uint64_t)u.num_clusters * u.num_features > (1u << 24))
        return fail(CKM_ERR_INVALID_ARGUMENT, "k*d too large");
    SJob* j = new SJob();
    j->u = u;
    j->t_submit = Clock::now();
    const bool large = (double)u.num_points * u.num_clusters * u.num_features >= (double)S->opt.large_work;
    j->bytes = large ? large_bytes(u) : small_layout(u.num_points, u.num_features, u.num_clusters).total;
    if (j->bytes > S->budget) {
        delete j;
        return fail(CKM_ERR_BUDGET, "job needs more device memory than the server's budget");
    }
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (S->stop) {
            delete j;
            return fail(CKM_ERR_INVALID_ARGUMENT, "server is stopping");
        }
        ++S->submitted;
        (large ? S->large_q : S->small_q).push_back(j);
    }
    S->cv_work.notify_all();
    return CKM_OK;
}

int ckm_server_poll(ckm_server* S, ckm_server_result* results, uint32_t max_results, uint32_t* count) {
    if (!S || !count || (max_results && !results)) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    const uint32_t m = (uint32_t)std::min<size_t>(max_results, S->results.size());
    for (uint32_t i = 0; i < m; ++i) results[i] = S->results[i];
    S->results.erase(S->results.begin(), S->results.begin() + m);
    *count = m;
    return CKM_OK;
}

int ckm_server_stats_get(ckm_server* S, ckm_server_stats* out) {
    if (!S || !out) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> g(S->mu);
    *out = S->stats;
    return CKM_OK;
}

int ckm_server_drain(ckm_server* S) {
    if (!S) return fail(CKM_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv_done.wait(lk, [&] { return S->completed == S->submitted; });
    return CKM_OK;
}

int ckm_server_destroy(ckm_server* S) {
    if (!S) return CKM_OK;
    ckm_server_drain(S);
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->small_thread.joinable()) S->small_thread.join();
    if (S->large_thread.joinable()) S->large_thread.join();
    {
        std::lock_guard<std::mutex> g(S->rmu);
        S->retire_stop = true;
    }
    S->cv_retire.notify_all();
    if (S->retire_thread.joinable()) S->retire_thread.join();
    for (cudaEvent_t ev : S->free_events) cudaEventDestroy(ev);
    cudaSetDevice(S->device);
    cudaDeviceSynchronize();
    for (int i = 0; i < 2; ++i) {
        ckm_batch_destroy(S->batch[i]);
        cudaFreeHost(S->h_status[i]);
        cudaEventDestroy(S->ev_status[i]);
        cudaEventDestroy(S->ev_s0[i]);
        cudaEventDestroy(S->ev_s1[i]);
    }
    cudaFree(S->d_status);
    cudaFree(S->d_tickets);
    cudaEventDestroy(S->ev_up);
    cudaStreamDestroy(S->s_up);
    cudaStreamDestroy(S->s_comp);
    cudaStreamDestroy(S->s_large);
    cudaStreamDestroy(S->s_down);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    delete S;
    return CKM_OK;
}

}  // extern "C"
