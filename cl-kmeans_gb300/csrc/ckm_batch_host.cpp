// Host side of the batched Lloyd iteration: the ckm_batch handle.
//
// create: uploads a device job table, allocates every job's FP64 scratch and
//         second centroid buffer in two arenas, and builds the work list:
//         every job's tiles cut into segments of similar estimated cost
//         (see build_schedule), largest first, claimed by the CTAs at run
//         time.  With autotune, candidate (tile size,
//         CTAs per SM) pairs are timed on the batch itself (two steps each,
//         with the device job state saved and restored around them).
// step:   one persistent kernel launch.
// run:    `iterations` steps; with use_graph the launches are captured once
//         into a CUDA graph per iteration count and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "ckm_batched.h"
#include "ckm_internal.h"

using namespace ckm;

struct ckm_batch {
    int device = 0;
    uint32_t num_jobs = 0;
    std::vector<ckm_batch_job> jobs;
    // device memory
    BatchJobDev* d_jobs = nullptr;
    BatchStatus* d_status = nullptr;
    unsigned int* d_tickets = nullptr;
    unsigned char* d_scratch = nullptr;   // per job: sums (8 k d) + msum (8 k), 256-aligned
    float* d_alt = nullptr;               // per job: second centroid buffer (4 k d)
    BatchSegment* d_segs = nullptr;
    unsigned int* d_work = nullptr;        // segments claimed in the current step
    // schedule
    uint32_t grid = 0, tile = 1024, ctas_per_sm = 1, block = 512, flush = 16, segments = 0;
    uint32_t use_umma = 0;                // d = 32 / 64 segments may use the tensor cores
    float tol = 0.f;                      // convergence stop (0: none)
    uint32_t max_it = 0;                  // iteration cap (0: none)
    uint32_t jobs_capacity = 0;           // entries of d_jobs
    size_t cent_cap = 0, acc_cap = 0;
    std::vector<BatchJobDev> host_dev_jobs;
    // graphs per iteration count
    std::map<uint32_t, cudaGraphExec_t> graphs;
    size_t seg_capacity = 0;
};

namespace {

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

int cuda_alloc(void** p, size_t bytes, const char* what) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, what);
}

// Builds the work list for (tile, grid): every job's tiles cut into segments
// of about 1/8 of a CTA's share of the estimated cost, largest first.  Cost
// per point: the distances (k*d) plus the shared-memory adds of the sums,
// which contend more the fewer clusters there are (d * (1 + 32/k) * 4), plus
// a constant.
void build_schedule(const std::vector<ckm_batch_job>& jobs, uint32_t tile, uint32_t grid,
                    std::vector<BatchSegment>& segs, std::vector<uint32_t>& tiles_per_job) {
    const uint32_t J = (uint32_t)jobs.size();
    tiles_per_job.assign(J, 0);
    double total = 0.0;
    std::vector<double> tile_cost(J, 0.0);
    for (uint32_t j = 0; j < J; ++j) {
        const ckm_batch_job& b = jobs[j];
        const double k = (double)b.num_clusters, d = (double)b.num_features;
        tiles_per_job[j] = (uint32_t)((b.num_points + tile - 1) / tile);
        tile_cost[j] = (double)tile * (k * d + 4.0 * d * (1.0 + 32.0 / k) + 32.0);
        total += tile_cost[j] * tiles_per_job[j];
    }
    const double unit = total / (8.0 * std::max<uint32_t>(grid, 1));
    std::vector<std::pair<double, BatchSegment>> units;
    for (uint32_t j = 0; j < J; ++j) {
        const uint32_t per = (uint32_t)std::max(1.0, std::floor(unit / std::max(tile_cost[j], 1.0)));
        for (uint32_t t = 0; t < tiles_per_job[j]; t += per) {
            const uint32_t te = std::min(tiles_per_job[j], t + per);
            units.push_back({tile_cost[j] * (te - t), BatchSegment{j, t, te, 0}});
        }
    }
    std::stable_sort(units.begin(), units.end(),
                     [](const std::pair<double, BatchSegment>& a, const std::pair<double, BatchSegment>& b) {
                         return a.first > b.first;
                     });
    segs.clear();
    segs.reserve(units.size());
    for (const auto& u : units) segs.push_back(u.second);
}

int upload_schedule(ckm_batch* b, uint32_t tile, uint32_t ctas_per_sm, cudaStream_t s) {
    const DeviceInfo& di = device_info();
    // shared-memory caps: the largest job's tables, bounded
    size_t need_c = 0, need_a = 0;
    for (const auto& j : b->jobs) {
        need_c = std::max(need_c, ((size_t)j.num_clusters * j.num_features + ((j.num_clusters + 3) & ~3u)) * sizeof(float));
        need_a = std::max(need_a, ((size_t)j.num_clusters * j.num_features + j.num_clusters) * sizeof(float));
    }
    const size_t budget = std::min<size_t>(di.smem_optin - 1024, 200 * 1024) / std::max<uint32_t>(ctas_per_sm, 1);
    // the rest holds the sum tables: one column per lane index (32 copies)
    // where a job's table fits that way, else one copy
    size_t cent_cap = std::min(a256(need_c), budget / 2);
    size_t acc_cap = std::min(a256(32 * need_a), budget - cent_cap);
    // one CTA per SM runs 512 threads (16 warps beside the whole shared
    // memory); two or more run 256 threads each
    const uint32_t block = ctas_per_sm <= 1 ? 512u : 256u;
    // the tensor-core path (d = 32 / 64; 512-thread CTAs, one per SM, 256
    // TMEM columns each) takes its operand tiles from the same budget, so a
    // batch with such jobs gets all of it
    bool umma_jobs = false;
    for (const auto& j : b->jobs)
        umma_jobs = umma_jobs || ((j.num_features == 32 || j.num_features == 64) &&
                                  j.num_clusters >= UMMA_MIN_K && j.num_clusters <= UMMA_MAX_K);
    const char* env = std::getenv("CKM_BATCH_UMMA");
    const bool umma_on = umma_jobs && block == 512 && !(env && env[0] == '0');
    if (umma_on) acc_cap = budget - cent_cap;
    int bps = 0;
    int st = batched_blocks_per_sm(cent_cap + acc_cap, block, &bps);
    if (st) return st;
    if (bps < 1) return fail(CKM_ERR_UNSUPPORTED, "batched kernel does not fit on an SM");
    const uint32_t cps = std::min<uint32_t>(std::max<uint32_t>(ctas_per_sm, 1), (uint32_t)bps);
    const uint32_t grid = (uint32_t)di.sm_count * cps;
    std::vector<BatchSegment> segs;
    std::vector<uint32_t> tiles;
    build_schedule(b->jobs, tile, grid, segs, tiles);
    if (segs.size() > b->seg_capacity) {
        if (b->d_segs) cudaFree(b->d_segs);
        b->d_segs = nullptr;
        b->seg_capacity = segs.size() + 64;
        if ((st = cuda_alloc((void**)&b->d_segs, b->seg_capacity * sizeof(BatchSegment), "cudaMalloc(segments)"))) return st;
    }
    if (!b->d_work && (st = cuda_alloc((void**)&b->d_work, sizeof(unsigned int), "cudaMalloc(work counter)"))) return st;
    cudaError_t e = cudaMemcpyAsync(b->d_segs, segs.data(), segs.size() * sizeof(BatchSegment), cudaMemcpyHostToDevice, s);
    for (uint32_t j = 0; j < b->num_jobs; ++j) b->host_dev_jobs[j].num_tiles = tiles[j];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_jobs, b->host_dev_jobs.data(), b->num_jobs * sizeof(BatchJobDev), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // host vectors go out of scope
    if (e != cudaSuccess) return cuda_fail(e, "upload schedule");
    b->grid = grid;
    b->tile = tile;
    b->ctas_per_sm = cps;
    b->block = block;
    b->segments = (uint32_t)segs.size();
    b->cent_cap = cent_cap;
    b->acc_cap = acc_cap;
    // CKM_BATCH_TEST_STALL=1 (tests only): the tensor-core waits run out, to
    // check that a failed job is reported
    const char* stall = std::getenv("CKM_BATCH_TEST_STALL");
    b->use_umma = umma_on ? (1u | ((stall && stall[0] == '1') ? 2u : 0u)) : 0u;
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
    b->graphs.clear();
    return CKM_OK;
}

int step(ckm_batch* b, cudaStream_t s) {
    return launch_batched(b->d_jobs, b->d_segs, b->segments, b->d_work, b->tol, b->max_it, b->grid, b->block, b->tile,
                          b->flush, b->cent_cap, b->acc_cap, b->use_umma, s);
}

int autotune(ckm_batch* b, cudaStream_t s) {
    // saved device job state, restored after every trial
    std::vector<BatchStatus> saved(b->num_jobs);
    cudaError_t e = cudaMemcpyAsync(saved.data(), b->d_status, b->num_jobs * sizeof(BatchStatus), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "autotune save");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    uint32_t best_tile = b->tile, best_cps = 1;
    const uint32_t tiles[] = {256, 1024, 4096};
    const uint32_t cpss[] = {1, 2, 4};
    int st = CKM_OK;
    for (uint32_t t : tiles) {
        for (uint32_t c : cpss) {
            if ((st = upload_schedule(b, t, c, s))) break;
            if (b->ctas_per_sm != c) continue;  // did not fit: already covered by a smaller count
            float ms_sum = 0.f;
            for (int rep = 0; rep < 2; ++rep) {
                cudaEventRecord(e0, s);
                if ((st = step(b, s))) break;
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep == 1) ms_sum += ms;  // first rep warms up
            }
            if (st) break;
            e = cudaMemcpyAsync(b->d_status, saved.data(), b->num_jobs * sizeof(BatchStatus), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                st = cuda_fail(e, "autotune restore");
                break;
            }
            if (ms_sum < best_ms) {
                best_ms = ms_sum;
                best_tile = t;
                best_cps = c;
            }
        }
        if (st) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    return upload_schedule(b, best_tile, best_cps, s);
}

void release(ckm_batch* b) {
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
    b->graphs.clear();
    cudaFree(b->d_jobs);
    cudaFree(b->d_status);
    cudaFree(b->d_tickets);
    cudaFree(b->d_scratch);
    cudaFree(b->d_alt);
    cudaFree(b->d_segs);
    cudaFree(b->d_work);
}

}  // namespace

extern "C" {

int ckm_batch_create(const ckm_batch_job* jobs, uint32_t num_jobs, const ckm_batch_options* options,
                     ckm_batch** out, ckm_stream_t stream) {
    if (!out) return fail(CKM_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (num_jobs == 0 || !jobs) return fail(CKM_ERR_INVALID_ARGUMENT, "no jobs");
    for (uint32_t j = 0; j < num_jobs; ++j) {
        const ckm_batch_job& b = jobs[j];
        if (b.num_features == 0 || b.num_clusters == 0)
            return fail(CKM_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": num_features/num_clusters must be >= 1");
        if (!b.centroids || !b.masses || (b.num_points && (!b.points || !b.labels)))
            return fail(CKM_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": NULL array");
        if ((uint64_t)b.num_clusters * b.num_features > (1u << 24))
            return fail(CKM_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": k*d too large for a batch");
        if (b.num_points > 0xffffffffull * 256ull)
            return fail(CKM_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + ": too many points");
    }
    cudaStream_t s = (cudaStream_t)stream;
    std::unique_ptr<ckm_batch> b(new ckm_batch());
    cudaGetDevice(&b->device);
    b->num_jobs = num_jobs;
    b->jobs.assign(jobs, jobs + num_jobs);
    ckm_batch_options opt{};
    if (options) opt = *options;
    b->flush = opt.flush_tiles ? opt.flush_tiles : 16;
    b->tol = opt.tolerance > 0.f ? opt.tolerance : 0.f;
    b->max_it = opt.max_iterations;
    b->jobs_capacity = num_jobs;
    // arenas
    size_t scratch_total = 0, alt_total = 0;
    std::vector<size_t> s_off(num_jobs), a_off(num_jobs);
    for (uint32_t j = 0; j < num_jobs; ++j) {
        const size_t kd = (size_t)jobs[j].num_clusters * jobs[j].num_features;
        s_off[j] = scratch_total;
        scratch_total += a256(kd * 8) + a256((size_t)jobs[j].num_clusters * 8);
        a_off[j] = alt_total;
        alt_total += a256(kd * 4);
    }
    int st;
    if ((st = cuda_alloc((void**)&b->d_jobs, num_jobs * sizeof(BatchJobDev), "cudaMalloc(job table)")) ||
        (st = cuda_alloc((void**)&b->d_status, num_jobs * sizeof(BatchStatus), "cudaMalloc(job status)")) ||
        (st = cuda_alloc((void**)&b->d_tickets, num_jobs * sizeof(unsigned int), "cudaMalloc(tickets)")) ||
        (st = cuda_alloc((void**)&b->d_scratch, scratch_total, "cudaMalloc(batch scratch)")) ||
        (st = cuda_alloc((void**)&b->d_alt, alt_total, "cudaMalloc(batch centroids)"))) {
        release(b.get());
        return st;
    }
    cudaError_t e = cudaMemsetAsync(b->d_status, 0, num_jobs * sizeof(BatchStatus), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_tickets, 0, num_jobs * sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_scratch, 0, scratch_total ? scratch_total : 16, s);
    if (e != cudaSuccess) {
        release(b.get());
        return cuda_fail(e, "cudaMemsetAsync(batch)");
    }
    b->host_dev_jobs.resize(num_jobs);
    for (uint32_t j = 0; j < num_jobs; ++j) {
        const ckm_batch_job& u = jobs[j];
        BatchJobDev& J = b->host_dev_jobs[j];
        const size_t kd = (size_t)u.num_clusters * u.num_features;
        J.points = u.points;
        J.cent[0] = u.centroids;
        J.cent[1] = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(b->d_alt) + a_off[j]);
        J.labels = u.labels;
        J.masses = u.masses;
        J.sums = reinterpret_cast<double*>(b->d_scratch + s_off[j]);
        J.msum = reinterpret_cast<unsigned long long*>(b->d_scratch + s_off[j] + a256(kd * 8));
        J.ticket = b->d_tickets + j;
        J.status = b->d_status + j;
        J.n = u.num_points;
        J.d = u.num_features;
        J.k = u.num_clusters;
        J.num_tiles = 0;
        J.pad = 0;
    }
    const uint32_t tile = opt.tile_points ? opt.tile_points : 1024;
    const uint32_t cps = opt.ctas_per_sm ? opt.ctas_per_sm : 1;
    if ((st = upload_schedule(b.get(), tile, cps, s))) {
        release(b.get());
        return st;
    }
    if (opt.autotune && !opt.tile_points && !opt.ctas_per_sm) {
        if ((st = autotune(b.get(), s))) {
            release(b.get());
            return st;
        }
    }
    *out = b.release();
    return CKM_OK;
}

int ckm_batch_step(ckm_batch* b, ckm_stream_t stream) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    return step(b, (cudaStream_t)stream);
}

int ckm_batch_sync(ckm_batch* b, ckm_stream_t stream) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    return launch_batch_sync(b->d_jobs, b->num_jobs, (cudaStream_t)stream);
}

int ckm_batch_run(ckm_batch* b, uint32_t iterations, int use_graph, ckm_stream_t stream) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    if (iterations == 0) return ckm_batch_sync(b, stream);
    if (!use_graph) {
        for (uint32_t i = 0; i < iterations; ++i) {
            int st = step(b, s);
            if (st) return st;
        }
        return ckm_batch_sync(b, stream);
    }
    auto it = b->graphs.find(iterations);
    if (it == b->graphs.end()) {
        // capture on a private stream, so the caller's stream may be the legacy one
        cudaStream_t cap = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate(capture)");
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            return cuda_fail(e, "cudaStreamBeginCapture");
        }
        int st = CKM_OK;
        for (uint32_t i = 0; i < iterations && st == CKM_OK; ++i) st = step(b, cap);
        if (st == CKM_OK) st = launch_batch_sync(b->d_jobs, b->num_jobs, cap);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        cudaGraphExec_t ge = nullptr;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        it = b->graphs.emplace(iterations, ge).first;
    }
    cudaError_t e = cudaGraphLaunch(it->second, s);
    count_launch(iterations + 1);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "cudaGraphLaunch");
}

int ckm_batch_status(ckm_batch* b, float* shifts, uint32_t* iterations, ckm_stream_t stream) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    std::vector<BatchStatus> st(b->num_jobs);
    cudaError_t e = cudaMemcpyAsync(st.data(), b->d_status, b->num_jobs * sizeof(BatchStatus), cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "ckm_batch_status");
    uint32_t failed = 0xffffffffu;
    for (uint32_t j = 0; j < b->num_jobs; ++j) {
        if (shifts) shifts[j] = st[j].shift;
        if (iterations) iterations[j] = st[j].iterations;
        if ((st[j].flags & 4u) && failed == 0xffffffffu) failed = j;
    }
    if (failed != 0xffffffffu)
        return fail(CKM_ERR_TIMEOUT, "batched: a wait for the tensor cores timed out (job " + std::to_string(failed) +
                                      " failed and is skipped by later steps)");
    return CKM_OK;
}

int ckm_batch_set_active(ckm_batch* b, const uint8_t* active, ckm_stream_t stream) {
    if (!b || !active) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<BatchStatus> st(b->num_jobs);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(st.data(), b->d_status, b->num_jobs * sizeof(BatchStatus), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "ckm_batch_set_active (read)");
    for (uint32_t j = 0; j < b->num_jobs; ++j) st[j].flags = active[j] ? (st[j].flags & ~1u) : (st[j].flags | 1u);
    e = cudaMemcpyAsync(b->d_status, st.data(), b->num_jobs * sizeof(BatchStatus), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? CKM_OK : cuda_fail(e, "ckm_batch_set_active (write)");
}

int ckm_batch_info(const ckm_batch* b, uint32_t* grid, uint32_t* tile_points, uint32_t* ctas_per_sm,
                   uint32_t* segments) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (grid) *grid = b->grid;
    if (tile_points) *tile_points = b->tile;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    if (segments) *segments = b->segments;
    return CKM_OK;
}

int ckm_batch_destroy(ckm_batch* b) {
    if (!b) return CKM_OK;
    cudaDeviceSynchronize();
    release(b);
    delete b;
    return CKM_OK;
}

}  // extern "C"

namespace ckm {

int batch_create_external(::ckm_batch** out) {
    if (!out) return fail(CKM_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = new ckm_batch();
    cudaGetDevice(&(*out)->device);
    return CKM_OK;
}

int batch_set_jobs(::ckm_batch* b, const BatchJobDev* jobs, uint32_t num_jobs, uint32_t tile, uint32_t ctas_per_sm,
                   float tol, uint32_t max_it, cudaStream_t s) {
    if (!b || (num_jobs && !jobs)) return fail(CKM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (num_jobs > b->jobs_capacity) {
        cudaFree(b->d_jobs);
        b->d_jobs = nullptr;
        b->jobs_capacity = num_jobs + 256;
        int st = cuda_alloc((void**)&b->d_jobs, b->jobs_capacity * sizeof(BatchJobDev), "cudaMalloc(job table)");
        if (st) {
            b->jobs_capacity = 0;
            return st;
        }
    }
    b->num_jobs = num_jobs;
    b->host_dev_jobs.assign(jobs, jobs + num_jobs);
    b->jobs.resize(num_jobs);
    for (uint32_t j = 0; j < num_jobs; ++j) {
        ckm_batch_job& u = b->jobs[j];
        std::memset(&u, 0, sizeof(u));
        u.num_points = jobs[j].n;
        u.num_features = jobs[j].d;
        u.num_clusters = jobs[j].k;
    }
    b->tol = tol;
    b->max_it = max_it;
    if (num_jobs == 0) {
        b->segments = 0;
        return CKM_OK;
    }
    return upload_schedule(b, tile, ctas_per_sm, s);
}

int batch_launch_step(::ckm_batch* b, cudaStream_t s) {
    if (!b) return fail(CKM_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (b->num_jobs == 0 || b->segments == 0) return CKM_OK;
    return step(b, s);
}

}  // namespace ckm
