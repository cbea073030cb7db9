"""Benchmark: Lloyd k-means iteration throughput on GB300 (points*iterations/s).

Workload (default): n = 2^28 points, d = 4 features, k = 16 clusters, float32,
column-major, from a 16-blob Gaussian mixture (centres U[-10,10]^4, sigma
U[0.5,2]), generated on the device from seed 42; initial centroids = first k
points.  One step = one Lloyd iteration over all points = ONE launch of the
fused kernel (label + mass + feature sums + FP64 merge + divide).

JSON line keys (rank 0):
  value      pts*it/s with the points resident in HBM (4 GiB > L2, so no L2
             flush is needed between steps)
  e2e        the same metric through the C ABI ckm_kmeans_run_f32 (the
             AbstractKmeans::operator() call) with pinned HOST buffers: every
             step copies the points in, runs the configured 50 iterations and
             copies centroids, labels and masses out
  roofline   HBM roofline of the fused kernel: algorithmic bytes per point-
             iteration = 4*d (points read once) + 4 (label written)
  cpu_baseline  the reference's own KmeansNaive32 (compiled unchanged into
             oracle/_ref; the oracle port where that build is absent) on a
             2^22-point sample of the same workload, one thread

--impl reference runs the reference's CPU path instead: its own KmeansNaive32
compiled unchanged (oracle/_ref; single-threaded, as the reference is) on a
bounded sample of the workload, with the oracle port threaded over all host
cores beside it.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (n, d, k, blobs, sigma_lo, sigma_hi, iterations of the configured run)
    "lloyd_n2^28_d4_k16": (1 << 28, 4, 16, 16, 0.5, 2.0, 50),
    "lloyd_n2^20_d4_k10": (1 << 20, 4, 10, 10, 1.0, 1.0, 30),
    # profiling-size case of the default workload: 160 MB of inputs (> L2)
    "lloyd_n2^25_d4_k16": (1 << 25, 4, 16, 16, 0.5, 2.0, 50),
}
DEFAULT_WORKLOAD = "lloyd_n2^28_d4_k16"
SEED = 42
FALLBACK_HBM_GBS = 6800.0


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                j = json.load(f)
            for key in ("hbm_gbs", "hbm_GBps", "hbm_copy_gbs"):
                if key in j and j[key]:
                    return float(j[key]), "measured"
        except (OSError, ValueError):
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic_per_point(key):
    """DRAM bytes per point-iteration of the fused kernel from the committed
    ncu summary's data file (profiles/fused_lowd_d4_k16.traffic.json), if any."""
    p = os.path.join(ROOT, "profiles", "fused_lowd_d4_k16.traffic.json")
    try:
        with open(p) as f:
            v = json.load(f).get(key)
        return float(v) if v is not None else None
    except (OSError, ValueError):
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    # where the raw samples go: $CKM_CLOCKS_CSV if set, else a temporary file
    def __init__(self, gpu_index):
        import tempfile
        self.gpu = gpu_index
        self.proc = None
        self.path = os.environ.get("CKM_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(),
                                                                     "ckm_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port_rate(P, n, d, k, iters, threads):
    """pts*it/s of the oracle's Lloyd on the given sample (wall clock)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    C0 = O.first_x_f32(P, n, d, k)
    t0 = time.perf_counter()
    if threads <= 1:
        O.lloyd_f32(P, n, d, k, iters, C0)
    else:
        O.lloyd_f32_mt(P, n, d, k, iters, C0, threads)
    dt = time.perf_counter() - t0
    return n * iters / dt, dt


def reference_cpu_available():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O.ref_available()


def reference_cpu_rate(P, n, d, k, iters):
    """pts*it/s of the reference's own KmeansNaive32 (kmeans_naive.cpp:31-106,
    compiled unchanged into oracle/_ref), single-threaded as the reference is,
    first-k initial centroids, timed over its iteration loop alone."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    C0 = O.first_x_f32(P, n, d, k)
    _, _, _, loop_s = O.ref_naive_f32_timed(P, n, d, k, iters, C0)
    return n * iters / loop_s, loop_s


def cpu_baseline_record(P, n, d, k, iters, what):
    """The CPU baseline of a bench line: the reference's own KmeansNaive32
    when oracle/_ref was built on this machine, else the oracle port."""
    if reference_cpu_available():
        rate, dt = reference_cpu_rate(P, n, d, k, iters)
        return {"value": rate, "unit": "pts*iter/s", "cores": 1, "host_cores": os.cpu_count(),
                "kind": "reference",
                "sample": "%s, %d iterations, %.1f s; KmeansNaive32 compiled unchanged, 1 of %d host cores"
                          % (what, iters, dt, os.cpu_count() or 1)}
    rate, dt = cpu_port_rate(P, n, d, k, iters, 1)
    return {"value": rate, "unit": "pts*iter/s", "cores": 1, "host_cores": os.cpu_count(), "kind": "port",
            "sample": "%s, %d iterations, %.1f s; oracle port (the reference build is absent on this machine)"
                      % (what, iters, dt)}


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    return O


def rel_err(C, R):
    """Normwise relative error max |C - R| / max |R| over entries finite in
    both (NaN marks an empty cluster)."""
    C = np.asarray(C, np.float64)
    R = np.asarray(R, np.float64)
    ok = np.isfinite(C) & np.isfinite(R)
    if not ok.any():
        return 0.0
    return float(np.abs(C[ok] - R[ok]).max() / max(float(np.abs(R[ok]).max()), 1e-300))


def fp64_means_check(P, n, d, k, labels, centroids, masses=None):
    """Centroids against the FP64 means of the same labels (the oracle's FP64
    sums), and whether the masses are the label counts."""
    O = oracle_module()
    sums, m64 = O.sums_f64(P, n, d, k, np.ascontiguousarray(labels, np.uint32))
    with np.errstate(invalid="ignore", divide="ignore"):
        ref = sums / np.tile(m64.astype(np.float64), d)
    out = {"max_rel_centroid_err_vs_fp64_means": rel_err(centroids, ref)}
    if masses is not None:
        out["masses_equal_label_counts"] = bool(np.array_equal(np.asarray(masses, np.uint64), m64))
    return out


def fp64_label_check(Xs, m, d, k, C_in, ours):
    """Labels of m sample points (column-major Xs) against the oracle's FP32
    labels (bit-exact expected) and its FP64 labels; a disagreement with FP64
    is explained when our label's FP64 distance exceeds the best one by no
    more than the FP32 distance rounding allows, (d + 4) 2^-24 relative."""
    O = oracle_module()
    ref32 = O.label_f32(Xs, m, d, k, C_in)
    lab64, _, _ = O.label_gap_f64(Xs, m, d, k, C_in)
    ours = np.asarray(ours, np.uint32)
    bad = np.nonzero(ours != lab64)[0]
    explained = 0
    if bad.size:
        X = np.asarray(Xs, np.float64).reshape(d, m)[:, bad].T
        Cr = np.asarray(C_in, np.float64).reshape(d, k).T
        Da = ((X - Cr[ours[bad]]) ** 2).sum(1)
        Db = ((X - Cr[lab64[bad]]) ** 2).sum(1)
        rho = (d + 4) * 2.0 ** -24
        explained = int(np.sum(Da - Db <= 2 * rho / (1 - rho) * Db + 1e-30))
    return {"sample_points": int(m), "label_mismatches_vs_fp32_oracle": int(np.sum(ours != ref32)),
            "label_mismatches_vs_fp64": int(bad.size), "fp64_mismatches_within_fp32_rounding": explained}


def host_sample(n_s, d, blobs, slo, shi):
    """A host-generated sample with the workload's distribution (numpy, same
    mixture parameters and seed), so the CPU arm touches no GPU code."""
    rng = np.random.default_rng(SEED)
    centres = rng.uniform(-10.0, 10.0, size=(blobs, d))
    sig = rng.uniform(slo, shi, size=blobs)
    comp = rng.integers(0, blobs, size=n_s)
    X = centres[comp] + sig[comp, None] * rng.standard_normal((n_s, d))
    return np.ascontiguousarray(X.astype(np.float32).T).reshape(-1)


def ranks_max_ms(total_ms, world):
    """The job's time over N replicas: the slowest rank's (an all-reduce MAX
    over the process group; world 1: the rank's own)."""
    if world <= 1:
        return total_ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(total_ms)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, max_ms):
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return units_per_rank * world / (max_ms / 1e3)


def run_reference_arm(args, workload):
    """The reference's own CPU implementation of the path: KmeansNaive32
    (kmeans_naive.cpp:31-106) compiled unchanged into oracle/_ref, which is
    single-threaded, so it runs on one of the host's cores.  One step = one
    Lloyd iteration over a bounded sample of the workload (host-generated,
    same mixture), the centroids carried from step to step; the value is the
    sample's points x steps over the reference's own loop time.  The oracle
    port threaded over all host cores is reported beside it."""
    n, d, k, blobs, slo, shi, iters_cfg = WORKLOADS[workload]
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    host_cores = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    have_ref = O.ref_available()
    # bounded sample, sized from a probe so warmup + steps take about a minute
    probe_n = 1 << 18
    P = host_sample(1 << 24, d, blobs, slo, shi)
    Pp = np.ascontiguousarray(P.reshape(d, -1)[:, :probe_n]).reshape(-1)
    if have_ref:
        rate, _ = reference_cpu_rate(Pp, probe_n, d, k, 2)
    else:
        rate, _ = cpu_port_rate(Pp, probe_n, d, k, 2, 1)
    budget_s = 60.0
    per_step_pts = max(1 << 14, min(1 << 24, int(rate * budget_s / max(1, args.steps + args.warmup))))
    n_s = 1 << int(np.floor(np.log2(per_step_pts)))
    Ps = np.ascontiguousarray(P.reshape(d, -1)[:, :n_s]).reshape(-1)
    C = O.first_x_f32(Ps, n_s, d, k)

    def one_step(C):
        if have_ref:
            C, _, _, loop_s = O.ref_naive_f32_timed(Ps, n_s, d, k, 1, C)
            return C, loop_s
        t0 = time.perf_counter()
        C, _, _ = O.lloyd_f32(Ps, n_s, d, k, 1, C)
        return C, time.perf_counter() - t0

    for _ in range(args.warmup):
        C, _ = one_step(C)
    loop_s = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        C, dt = one_step(C)
        loop_s += dt
    wall = time.perf_counter() - t0
    value = n_s * args.steps / loop_s
    kind = "reference" if have_ref else "port"
    impl = ("KmeansNaive32 (kmeans_naive.cpp) compiled unchanged (oracle/_ref), single-threaded" if have_ref else
            "oracle port of KmeansNaive (the reference build is absent on this machine), single-threaded")
    # the port threaded over every host core, one iteration on the same sample
    Cp = O.first_x_f32(Ps, n_s, d, k)
    tp = time.perf_counter()
    O.lloyd_f32_mt(Ps, n_s, d, k, 1, Cp, host_cores)
    port_mt = n_s / (time.perf_counter() - tp)
    line = {
        "impl": "reference", "metric": "pts*iter/s", "value": value, "unit": "pts*iter/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": loop_s / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Gaussian mixture, host-generated sample of the workload)",
        "config": {"workload": workload, "n": n, "d": d, "k": k, "sample_points": n_s, "implementation": impl},
        "cpu_baseline": {"value": value, "unit": "pts*iter/s", "cores": 1, "host_cores": host_cores, "kind": kind,
                         "sample": "%d points of the workload, 1 iteration per step, %d steps, %.1f s wall"
                                   % (n_s, args.steps, wall)},
        "e2e": {"value": value, "unit": "pts*iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "port_threaded": {"value": port_mt, "unit": "pts*iter/s", "cores": host_cores,
                          "call": "oracle port of KmeansNaive, labeling and sums split over host threads"},
    }
    print(json.dumps(line), flush=True)
    return 0


def make_batched_jobs(ckm, torch, num_jobs, seed_base, dev):
    """Batched-jobs workload: per job n log-uniform in [2^10, 2^18], d from
    {2, 8, 32, 64}, k log-uniform in [4, 256] with k <= n/16, its own mixture
    of k blobs (centres U[-10,10]^d, sigma 1) from seed base + job id,
    initial centroids = first k points."""
    rng = np.random.default_rng(seed_base)
    jobs = []
    for j in range(num_jobs):
        n = int(round(np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 18)))))
        d = int(rng.choice([2, 8, 32, 64]))
        k = int(round(np.exp(rng.uniform(np.log(4), np.log(256)))))
        k = max(1, min(k, n // 16))
        P = torch.empty(n * d, dtype=torch.float32, device=dev)
        ckm.generate_mixture(P, n, d, k, seed_base + j, sigma=(1.0, 1.0))
        C0 = P.view(d, n)[:, :k].reshape(-1).clone()
        jobs.append(dict(points=P, centroids=C0.clone(), init=C0,
                         labels=torch.empty(n, dtype=torch.int32, device=dev),
                         masses=torch.empty(k, dtype=torch.int32, device=dev), n=n, d=d, k=k))
    return jobs


def batched_record(ckm, torch, dev, num_jobs, steps, warmup, fp64=True):
    """Batched uneven jobs: every job 20 fixed iterations, all jobs advanced by
    one persistent launch per iteration (CUDA graph), against the plain
    per-job loop (each job: its own fused launch per iteration) on the same
    GPU.  Metric: jobs/s.  Returns the record."""
    iters = 20
    jobs = make_batched_jobs(ckm, torch, num_jobs, 1234, dev)
    total_pts = sum(j["n"] for j in jobs)
    stream = torch.cuda.current_stream()
    # plain per-job loop (the reference's one-problem-at-a-time structure):
    # ckm_fused_f32 per job and iteration, called through the raw C ABI with
    # the pointers prepared once, so the loop's cost is the per-job call and
    # its launches, not Python argument handling
    scratch = {}
    alt = [torch.empty_like(j["centroids"]) for j in jobs]
    fn = ckm.lib().ckm_fused_f32
    s_arg = ctypes.c_void_p(stream.cuda_stream)
    calls = []
    for j, a in zip(jobs, alt):
        key = (j["d"], j["k"])
        if key not in scratch:
            scratch[key] = ckm.new_scratch(j["d"], j["k"], dev)
        sc = scratch[key]
        calls.append((j["d"], j["n"], j["k"], j["points"].data_ptr(), (j["centroids"].data_ptr(), a.data_ptr()),
                      j["labels"].data_ptr(), j["masses"].data_ptr(), sc.data_ptr(), sc.numel()))
    mode = ckm.MODE_FINALIZE

    def plain_all():
        for d_, n_, k_, P_, C_, L_, M_, S_, SN_ in calls:
            for it in range(iters):
                rc = fn(d_, n_, k_, P_, C_[it & 1], C_[(it + 1) & 1], L_, M_, S_, SN_, mode, s_arg)
                if rc:
                    ckm.check(rc, "ckm_fused_f32")

    for j in jobs:
        j["centroids"].copy_(j["init"])
    plain_all()  # warm-up (also allocates scratch)
    for j in jobs:
        j["centroids"].copy_(j["init"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_all()
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_result = [(a if iters % 2 else j["centroids"]).clone() for j, a in zip(jobs, alt)]

    # batched: one persistent launch per iteration, captured in a graph
    for j in jobs:
        j["centroids"].copy_(j["init"])
    batch = ckm.Batch(jobs, autotune=True)
    info = batch.info()
    warm = max(3, warmup)
    for _ in range(warm):                 # capture + warm-up
        for j in jobs:
            j["centroids"].copy_(j["init"])
        batch.run(iters, use_graph=True)
    times = []
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    for _ in range(max(3, steps if steps < 20 else 5)):
        for j in jobs:
            j["centroids"].copy_(j["init"])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches0 = ckm.launch_count()
        e0.record(stream)
        batch.run(iters, use_graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        gpu_launches = ckm.launch_count() - launches0
    clocks = sampler.stop()
    batch_s = statistics.median(times)
    # agreement with the plain loop after 20 iterations (same arithmetic;
    # FP64-merged sums in another order)
    worst, diverged = 0.0, 0
    for j, ref in zip(jobs, plain_result):
        e = rel_err(j["centroids"].cpu().numpy(), ref.cpu().numpy())
        worst = max(worst, e)
        diverged += e > 1e-5
    fp64_e2e = None
    if fp64:
        # 20 iterations end to end against the FP64 oracle (FP64 distances and
        # sums on the same FP32 points, the same start), on the jobs small
        # enough for the CPU; the oracle's own FP32 run (the reference's
        # arithmetic) beside it shows how far FP32 Lloyd itself drifts
        O = oracle_module()
        small = [i for i, j in enumerate(jobs) if j["n"] * j["k"] * j["d"] <= (1 << 20)][:32]
        errs, ref_errs = [], []
        for i in small:
            j = jobs[i]
            Ph = j["points"].cpu().numpy()
            C64, _, _ = O.lloyd_fp64_of_f32(Ph, j["n"], j["d"], j["k"], iters, j["init"].cpu().numpy())
            C32, _, _ = O.lloyd_f32(Ph, j["n"], j["d"], j["k"], iters, j["init"].cpu().numpy())
            errs.append(rel_err(j["centroids"].cpu().numpy(), C64))
            ref_errs.append(rel_err(C32, C64))
        fp64_e2e = {"jobs": len(small), "max_rel_centroid_err": max(errs) if errs else None,
                    "jobs_within_1e-5": int(sum(e <= 1e-5 for e in errs)),
                    "reference_fp32_max_rel_err": max(ref_errs) if ref_errs else None,
                    "reference_fp32_jobs_within_1e-5": int(sum(e <= 1e-5 for e in ref_errs)),
                    "selection": "jobs with n*k*d <= 2^20 (the first 32)"}
    # lockstep: one iteration of every job from the same centroids, batched
    # against the plain fused call and against the FP64 oracle
    for j in jobs:
        j["centroids"].copy_(j["init"])
    batch.run(1, use_graph=False)
    lock_worst, lock_label_diff = 0.0, 0
    for j, a in zip(jobs, alt):
        key = (j["d"], j["k"])
        lab = torch.empty_like(j["labels"])
        mas = torch.empty_like(j["masses"])
        ckm.fused(j["points"], j["init"], a, lab, mas, scratch[key], j["n"], j["d"], j["k"], ckm.MODE_FINALIZE, stream)
        torch.cuda.synchronize()
        lock_label_diff += int((lab != j["labels"]).sum().item())
        lock_worst = max(lock_worst, rel_err(j["centroids"].cpu().numpy(), a.cpu().numpy()))
    lock64 = None
    if fp64:
        O = oracle_module()
        sample = list(range(0, len(jobs), max(1, len(jobs) // 256)))
        worst64, masses_ok, lab_mis, lab_jobs = 0.0, True, 0, 0
        for i in sample:
            j = jobs[i]
            Ph = j["points"].cpu().numpy()
            labels = j["labels"].cpu().numpy().view(np.uint32)
            r = fp64_means_check(Ph, j["n"], j["d"], j["k"], labels, j["centroids"].cpu().numpy(),
                                 j["masses"].cpu().numpy().view(np.uint32))
            worst64 = max(worst64, r["max_rel_centroid_err_vs_fp64_means"])
            masses_ok &= r["masses_equal_label_counts"]
            if j["n"] * j["k"] * j["d"] <= (1 << 23) and lab_jobs < 64:
                lab_jobs += 1
                lab_mis += int(np.sum(O.label_f32(Ph, j["n"], j["d"], j["k"], j["init"].cpu().numpy()) != labels))
        lock64 = {"jobs": len(sample), "max_rel_centroid_err_vs_fp64_means": worst64,
                  "within_1e-5": bool(worst64 <= 1e-5), "masses_equal_label_counts": bool(masses_ok),
                  "label_mismatches_vs_fp32_oracle": lab_mis, "label_checked_jobs": lab_jobs}
    batch.close()
    flops = sum(2.0 * j["n"] * j["k"] * j["d"] for j in jobs) * iters
    algo_bytes = sum(float(j["n"]) * (4 * j["d"] + 4) for j in jobs) * iters
    peak, peak_kind = measured_hbm_peak()
    achieved = algo_bytes / batch_s / 1e9
    return {
        "metric": "jobs/s", "value": num_jobs / batch_s, "unit": "jobs/s", "n_gpus": 1, "steps": len(times),
        "warmup": warm, "ms_per_step": batch_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (per-job seeded Gaussian mixtures generated on the device)",
        "config": {"workload": "batched_%d_jobs" % num_jobs, "iterations": iters, "total_points": total_pts,
                   "schedule": info, "graph": True},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None, "algorithmic_bytes_per_step": algo_bytes},
        "tflops_exact_equivalent": flops / batch_s / 1e12,
        "plain_per_job_loop": {"jobs_per_s": num_jobs / plain_s, "seconds": plain_s,
                               "launches": num_jobs * iters},
        "speedup_vs_plain_loop": plain_s / batch_s,
        "pts_iter_per_s": total_pts * iters / batch_s,
        "lockstep_vs_plain": {"max_rel_centroid_diff": lock_worst, "label_mismatches": lock_label_diff},
        "lockstep_vs_fp64": lock64,
        "after_20_iterations_vs_plain": {"max_rel_centroid_diff": worst, "jobs_beyond_1e-5": int(diverged)},
        "after_20_iterations_vs_fp64": fp64_e2e,
        "gpu_launches": int(gpu_launches), "clocks": clocks,
    }


def run_batched_workload(args, ckm, torch, dev):
    if args.batch_d or args.batch_min_k or args.batch_max_k or args.batch_max_jobs or args.no_plain:
        # a class of the same job list (profiling and breakdowns): the
        # batched launches alone
        jobs = make_batched_jobs(ckm, torch, args.jobs, 1234, dev)
        jobs = [j for j in jobs if (not args.batch_d or j["d"] == args.batch_d) and j["k"] >= args.batch_min_k
                and (not args.batch_max_k or j["k"] < args.batch_max_k)]
        if args.batch_max_jobs:
            jobs = jobs[:args.batch_max_jobs]
        subset = {"d": args.batch_d or None, "min_k": args.batch_min_k, "max_k": args.batch_max_k or None,
                  "of_jobs": args.jobs}
        torch.cuda.empty_cache()
        return run_batched_only(args, ckm, torch, jobs, 20, sum(j["n"] for j in jobs), subset,
                                torch.cuda.current_stream())
    print(json.dumps(batched_record(ckm, torch, dev, args.jobs, args.steps, args.warmup)), flush=True)
    return 0


def run_batched_only(args, ckm, torch, jobs, iters, total_pts, subset, stream):
    """--no-plain: the batched launches alone (one step = one iteration of
    every job, no graph), for profiling a class of jobs."""
    batch = ckm.Batch(jobs, tile_points=4096, ctas_per_sm=1)
    warm = max(3, args.warmup)
    for _ in range(warm):
        batch.step(stream)
    torch.cuda.synchronize()
    steps = max(1, args.steps if args.steps < 1000 else 5)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ckm.launch_count()
    e0.record(stream)
    for _ in range(steps):
        batch.step(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    gpu_launches = ckm.launch_count() - launches0
    info = batch.info()
    batch.close()
    work = sum(j["n"] * j["k"] * j["d"] * 2 for j in jobs)
    line = {
        "metric": "pts*iter/s", "value": total_pts / (ms / 1e3), "unit": "pts*iter/s", "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (per-job seeded Gaussian mixtures generated on the device)",
        "config": {"workload": "batched_%d_jobs_one_iteration" % len(jobs), "subset": subset,
                   "total_points": total_pts, "schedule": info, "graph": False},
        "exact_arithmetic_tflops": work / ms / 1e9,
        "gpu_launches": int(gpu_launches),
    }
    print(json.dumps(line), flush=True)
    return 0


def host_mem_available():
    """MemAvailable of this host in bytes (None if /proc/meminfo is unreadable)."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except (OSError, ValueError):
        pass
    return None


def buffered_record(ckm, torch, dev, n, budget, iters, steps):
    """Out-of-core Lloyd (config 2b): n = 2^31 points of d = 16 from a 64-blob
    mixture (centres U[-10,10]^16, sigma U[0.5,2]) held in PINNED HOST memory
    (128 GiB), k = 64, first_x initial centroids, run through the buffered
    three-stage pipeline (ckm_kmeans_run_f32, three_stage_buffered) with the
    device budget capped at 32 GiB, so most chunks stream over the host link
    every iteration; 50 iterations.  Metric: pts*iter/s end to end (host
    points, device compute, host labels).  The host must hold the points and
    labels pinned with room to spare: the run is refused, with the measured
    figures, when MemAvailable is below that."""
    d, k, blobs = 16, 64, 64
    budget = budget or min((n * d * 4) // 4, 32 << 30)
    need = n * d * 4 + n * 4
    avail = host_mem_available()
    margin = 24 << 30
    if avail is not None and avail < need + margin:
        return {"metric": "pts*iter/s", "unit": "pts*iter/s", "n_gpus": 1,
                "config": {"workload": "buffered_three_stage_n%d_d%d_k%d" % (n, d, k)},
                "unavailable": "host MemAvailable %.1f GiB < %.1f GiB of pinned points and labels + "
                               "%.0f GiB margin" % (avail / 2 ** 30, need / 2 ** 30, margin / 2 ** 30)}
    # host points generated on the device in chunks of the same mixture
    P = torch.empty(n * d, dtype=torch.float32, pin_memory=True)
    L = torch.empty(n, dtype=torch.int32, pin_memory=True)
    chunk = 1 << 25
    buf = torch.empty(chunk * d, dtype=torch.float32, device=dev)
    Pv = P.view(d, n)
    for p0 in range(0, n, chunk):
        m = min(chunk, n - p0)
        ckm.generate_mixture(buf, m, d, blobs, SEED, sigma=(0.5, 2.0), first_point=p0)
        Pv[:, p0:p0 + m].copy_(buf[:m * d].view(d, m), non_blocking=False)
    del buf
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    Pn, Ln = P.numpy(), L.numpy().view(np.uint32)
    C0 = np.ascontiguousarray(Pv[:, :k].numpy()).reshape(-1)
    link = ckm.transfer_probe(1 << 30, repeat=4, pinned=True, to_device=True, trials=2)

    def run(iterations):
        t0 = time.perf_counter()
        C, M, Lo, info = ckm.kmeans_run(Pn, d, k, iterations, C0, pipeline="three_stage_buffered",
                                        device_budget_bytes=budget, labels=Ln)
        return time.perf_counter() - t0, info, M

    run(1)                          # warm-up: allocations, first chunks
    times, infos = [], []
    steps = max(1, min(steps, 3))
    for _ in range(steps):
        t, info, M = run(iters)
        times.append(t)
        infos.append(info)
    t = statistics.median(times)
    info = infos[0]
    assert int(M.astype(np.uint64).sum()) == n
    line = {
        "metric": "pts*iter/s", "value": n * iters / t, "unit": "pts*iter/s", "n_gpus": 1, "steps": steps,
        "warmup": 1, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded 64-blob mixture generated on the device, copied to pinned host memory)",
        "config": {"workload": "buffered_three_stage_n%d_d%d_k%d" % (n, d, k), "n": n, "d": d, "k": k,
                   "iterations_per_step": iters, "point_bytes": n * d * 4, "device_budget_bytes": budget,
                   "pipeline": "three_stage_buffered", "host_memory": "pinned"},
        "h2d_bytes_per_step": int(info.h2d_bytes), "d2h_bytes_per_step": int(info.d2h_bytes),
        "h2d_gbs_effective": info.h2d_bytes / t / 1e9,
        "h2d_link_probe_gbs": link[0],
        "kernel_launches_per_step": int(info.kernel_launches),
        "host_mem_available_gib": avail / 2 ** 30 if avail is not None else None,
    }
    del P, L, Pn, Ln
    return line


def run_buffered_workload(args, ckm, torch, dev):
    rec = buffered_record(ckm, torch, dev, args.buffered_points or (1 << 31), args.buffered_budget,
                          args.buffered_iterations, args.steps)
    print(json.dumps(rec), flush=True)
    return 0


def measured_bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                j = json.load(f)
            for key in ("bf16_tflops", "bf16_tflops_burst"):
                if key in j and j[key]:
                    return float(j[key]), "measured"
        except (OSError, ValueError):
            pass
    return 1900.0, "fallback"


def serving_record(ckm, torch, dev, seconds, rate, large_rate, pool_size, plain_jobs, round_iterations,
                   with_70pct=True, burst_rounds=4, fp64=True):
    """Served stream (config 5, scaled to what one GB300 and its host link
    carry): Poisson arrivals of config-4-shaped jobs (n log-U[2^10, 2^18],
    d in {2, 8, 32, 64}, k log-U[4, 256], k <= n/16) at `rate` jobs/s for
    `seconds`, plus large jobs (n = 2^22, d = 128, k = 1024) at `large_rate`
    jobs/s; every job stops at relative centroid shift < 1e-4 or 50
    iterations.  Payloads come from pools generated once and held in pinned
    host memory.  Reports throughput and p50/p99 latency under the stream,
    the burst capacity of the batched lane, and a plain per-job loop
    (ckm_kmeans_run with convergence, one job at a time) on the same jobs.
    Returns the record."""
    rng = np.random.default_rng(2024)
    tol, cap = 1e-4, 50
    # small-job pool
    pool = []
    for i in range(pool_size):
        n = int(round(np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 18)))))
        d = int(rng.choice([2, 8, 32, 64]))
        k = int(round(np.exp(rng.uniform(np.log(4), np.log(256)))))
        k = max(1, min(k, n // 16))
        P = torch.empty(n * d, dtype=torch.float32, device=dev)
        ckm.generate_mixture(P, n, d, k, 5000 + i, sigma=(1.0, 1.0))
        hp = torch.empty(n * d, dtype=torch.float32, pin_memory=True)
        hp.copy_(P)
        C0 = np.ascontiguousarray(hp.numpy().reshape(d, n)[:, :k]).reshape(-1)
        pool.append((hp, hp.numpy(), C0, n, d, k))
        del P
    large = []
    if large_rate > 0:
        for i in range(2):
            n, d, k = 1 << 22, 128, 1024
            P = torch.empty(n * d, dtype=torch.float32, device=dev)
            ckm.generate_mixture_ex(P, n, d, k, 9000 + i, center=("normal", 0.0, 2.0), sigma=("loguniform", 0.25, 1.0),
                                    dirichlet=True)
            hp = torch.empty(n * d, dtype=torch.float32, pin_memory=True)
            hp.copy_(P)
            C0 = np.ascontiguousarray(hp.numpy().reshape(d, n)[:, :k]).reshape(-1)
            large.append((hp, hp.numpy(), C0, n, d, k))
            del P
    torch.cuda.synchronize()

    def submit(S, item, tag):
        _, P, C0, n, d, k = item
        S.submit(P, C0, n, d, k, tag)

    def stream(lam, lam_l, T, seed):
        r2 = np.random.default_rng(seed)
        arrivals = []
        t = 0.0
        while True:
            t += r2.exponential(1.0 / lam)
            if t > T:
                break
            arrivals.append((t, 0))
        t = 0.0
        while lam_l > 0:
            t += r2.exponential(1.0 / lam_l)
            if t > T:
                break
            arrivals.append((t, 1))
        arrivals.sort()
        S = ckm.Server(tolerance=tol, max_iterations=cap, large_work=1 << 33, round_iterations=round_iterations)
        results = []
        t0 = time.perf_counter()
        for i, (ta, kind) in enumerate(arrivals):
            now = time.perf_counter() - t0
            if ta > now:
                time.sleep(ta - now)
            item = large[i % len(large)] if kind else pool[i % len(pool)]
            submit(S, item, i)
            if i % 64 == 0:
                results += S.poll()
        S.drain()
        t_end = time.perf_counter() - t0
        while True:
            more = S.poll()
            if not more:
                break
            results += more
        S.close()
        ok = [r for r in results if r["status"] == 0]
        lat_s = np.array([r["latency_ns"] for r in ok if r["lane"] == 0]) / 1e6
        lat_l = np.array([r["latency_ns"] for r in ok if r["lane"] != 0]) / 1e6
        its = np.array([r["iterations"] for r in ok if r["lane"] == 0])
        pct = lambda a, q: float(np.percentile(a, q)) if a.size else None
        summary = {"offered_small_per_s": lam, "offered_large_per_s": lam_l, "seconds": T,
                   "offered_jobs": len(arrivals), "completed_ok": len(ok), "failed": len(results) - len(ok),
                   "jobs_per_s": len(ok) / t_end,
                   "latency_ms_small": {"p50": pct(lat_s, 50), "p99": pct(lat_s, 99)},
                   "latency_ms_large": {"p50": pct(lat_l, 50), "p99": pct(lat_l, 99), "count": int(lat_l.size)},
                   "iterations_small_mean": float(its.mean()) if its.size else None,
                   "converged_fraction_small": float(np.mean([r["converged"] for r in ok if r["lane"] == 0]))
                   if its.size else None}
        return summary, ok

    # burst capacity of the batched lane: the whole small pool, several times over, at once
    S = ckm.Server(tolerance=tol, max_iterations=cap, large_work=1 << 33, round_iterations=round_iterations)
    nb = burst_rounds * len(pool)
    tb = time.perf_counter()
    for i in range(nb):
        submit(S, pool[i % len(pool)], i)
        if i % 256 == 0:
            S.poll()
    S.drain()
    burst_s = time.perf_counter() - tb
    while S.poll():
        pass
    burst_stats = S.stats()
    S.close()

    # plain per-job loop on the same small jobs (public host-level call)
    nplain = min(len(pool), plain_jobs)
    tp = time.perf_counter()
    for i in range(nplain):
        _, P, C0, n, d, k = pool[i]
        ckm.kmeans_run(P, d, k, cap, C0, converge=True, tolerance=tol)
    plain_s = (time.perf_counter() - tp) / nplain

    cap_rate = nb / burst_s
    sampler = ClockSampler(0)
    sampler.start()
    spec, ok = stream(rate, large_rate, seconds, 7)
    clocks = sampler.stop()
    sustain = None
    if with_70pct:
        # moderate load: 70 % of the configured small-job rate, same large jobs
        # (the burst capacity ignores the device time the large jobs take)
        sustain, _ = stream(0.7 * rate, large_rate, seconds, 8)
    check = None
    if fp64:
        # served small jobs: centroids against the FP64 means of the labels
        # they were returned with, masses against the label counts
        worst, masses_ok, nchk = 0.0, True, 0
        for r in ok:
            if r["lane"] != 0 or nchk >= 64:
                continue
            _, P, _, n, d, k = pool[r["tag"] % len(pool)]
            c = fp64_means_check(P, n, d, k, r["labels"], r["centroids"], r["masses"])
            worst = max(worst, c["max_rel_centroid_err_vs_fp64_means"])
            masses_ok &= c["masses_equal_label_counts"]
            nchk += 1
        check = {"jobs": nchk, "max_rel_centroid_err_vs_fp64_means": worst, "within_1e-5": bool(worst <= 1e-5),
                 "masses_equal_label_counts": bool(masses_ok)}
    return {
        "metric": "jobs/s", "value": spec["jobs_per_s"], "unit": "jobs/s", "n_gpus": 1, "steps": spec["offered_jobs"],
        "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (large jobs: fp16 tensor-core distances, exact FP32 labels)",
        "data": "synthetic (seeded mixtures, pinned host payload pools)",
        "config": {"workload": "served_stream", "seconds": seconds, "small_rate_per_s": rate,
                   "large_rate_per_s": large_rate, "small_pool": len(pool), "tolerance": tol,
                   "max_iterations": cap, "round_iterations": round_iterations or 4},
        "latency_ms_small": spec["latency_ms_small"],
        "stream_at_config_rate": spec,
        "stream_at_70pct_config_rate": sustain,
        "burst_capacity_small_jobs_per_s": cap_rate,
        "burst_lane_stats": dict(burst_stats, wall_ns=int(burst_s * 1e9)),
        "plain_per_job_loop": {"jobs_per_s": 1.0 / plain_s, "jobs": nplain,
                               "call": "ckm_kmeans_run_f32(single_stage, converge) per job"},
        "capacity_vs_plain_loop": cap_rate * plain_s,
        "fp64_check": check, "clocks": clocks,
    }


def run_serving_workload(args, ckm, torch, dev):
    rec = serving_record(ckm, torch, dev, args.serve_seconds, args.serve_rate, args.serve_large_rate, args.serve_pool,
                         args.serve_plain_jobs, args.serve_round)
    print(json.dumps(rec), flush=True)
    return 0


def tensor_core_record(ckm, torch, dev, n, steps, warmup, simt_compare=True, cpu_baseline=True, fp64=True,
                       precision="fp16"):
    """Tensor-core labeling with precision recovery: n = 2^24, d = 128,
    k = 1024, a 1024-component mixture (centres ~ N(0, 4 I), sigma
    log-uniform in [0.25, 1], Dirichlet(1) weights), 20 fixed iterations.
    One step = one Lloyd iteration via ckm_tc_fused_f32 (fp16 distance GEMM
    on tcgen05, certified labels, exact FP32 recheck of near-ties, FP64
    sums).  Returns the record (a JSON-able dict)."""
    d, k, iters = 128, 1024, 20
    stream = torch.cuda.current_stream()
    P = torch.empty(n * d, dtype=torch.float32, device=dev)
    ckm.generate_mixture_ex(P, n, d, k, SEED, center=("normal", 0.0, 2.0), sigma=("loguniform", 0.25, 1.0),
                            dirichlet=True)
    tcp = ckm.TensorCorePoints(P, n, d, precision=precision)
    C = [P.view(d, n)[:, :k].reshape(-1).clone(), torch.empty(k * d, dtype=torch.float32, device=dev)]
    C0 = C[0].clone()
    L = torch.empty(n, dtype=torch.int32, device=dev)
    M = torch.empty(k, dtype=torch.int32, device=dev)
    S = ckm.new_scratch(d, k, dev)
    stats = torch.zeros(2, dtype=torch.int32, device=dev)
    steps = min(steps, iters)
    warm = max(3, min(warmup, 5))
    for i in range(warm):
        ckm.tc_fused(P, tcp, C[i % 2], C[(i + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stats, stream)
        if i == 0:
            tcp.sort(k, stream)  # cluster-ordered tiles from the first labels (once per run)
    C[0].copy_(C0)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    rechecked, resolved, overflowed = [], [], []
    counters = torch.zeros(4, dtype=torch.int32, device=dev)
    launches0 = ckm.launch_count()
    for i in range(steps):
        evs[i][0].record(stream)
        ckm.tc_fused(P, tcp, C[i % 2], C[(i + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stats, stream)
        evs[i][1].record(stream)
        torch.cuda.synchronize()
        tcp.counters(k, counters, stream)
        st = counters.cpu().numpy()
        rechecked.append(int(st[0]))
        resolved.append(int(st[2]))
        overflowed.append(int(st[3]))
        if st[1]:
            raise RuntimeError("tensor-core kernel reported a timed-out device wait")
    gpu_launches = ckm.launch_count() - launches0
    clocks = sampler.stop()
    ms = [a.elapsed_time(b) for a, b in evs]
    step_s = statistics.mean(ms) / 1e3
    flops = 2.0 * n * k * d
    peak, kind = measured_bf16_peak()
    achieved = flops / step_s / 1e12
    check = None
    if fp64:
        # the last step against the FP64 oracle: its labels on a sample of
        # points from the same input centroids, and its centroids against
        # the FP64 means of its labels over all points
        C_in = C[(steps - 1) % 2].cpu().numpy()
        C_out = C[steps % 2].cpu().numpy()
        labels = L.cpu().numpy().view(np.uint32)
        Ph = P.cpu().numpy()
        rng = np.random.default_rng(5)
        sample = np.sort(rng.choice(n, size=min(n, 1 << 13), replace=False))
        Xs = np.ascontiguousarray(Ph.reshape(d, n)[:, sample]).reshape(-1)
        check = fp64_label_check(Xs, len(sample), d, k, C_in, labels[sample])
        check.update(fp64_means_check(Ph, n, d, k, labels, C_out, M.cpu().numpy().view(np.uint32)))
        del Ph
    # the same iteration on the FP32 SIMT path (exact arithmetic everywhere), one step
    simt_s = None
    if simt_compare:
        Ls = torch.empty(n, dtype=torch.int32, device=dev)
        Cs = torch.empty(k * d, dtype=torch.float32, device=dev)
        Ss = ckm.new_scratch(d, k, dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ckm.fused(P, C0, Cs, Ls, M, Ss, n, d, k, ckm.MODE_FINALIZE, stream)
        torch.cuda.synchronize()
        simt_s = time.perf_counter() - t0
    cpu = None
    if cpu_baseline:
        n_s = 1 << 12
        Ps = np.ascontiguousarray(P.view(d, n)[:, :n_s].cpu().numpy()).reshape(-1)
        cpu = cpu_baseline_record(Ps, n_s, d, k, 1, "first %d points" % n_s)
    return {
        "metric": "pts*iter/s", "value": n / step_s, "unit": "pts*iter/s", "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "%s distances (tcgen05), f32 exact candidates, f64 sums" % precision,
        "data": "synthetic (seeded 1024-component mixture generated on the device)",
        "config": {"workload": "lloyd_tc_n%d_d%d_k%d" % (n, d, k), "n": n, "d": d, "k": k,
                   "centres": "N(0, 4I)", "sigma": "log-uniform [0.25, 1]", "weights": "Dirichlet(1)",
                   "point_order": "sorted by cluster once, after the first iteration (ckm_tc_sort_points)",
                   "l2": "inputs (%.1f GiB) larger than L2, no flush" % (n * d * 6 / 2 ** 30)},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_source": kind, "traffic": None,
                     "algorithmic_flops_per_step": flops},
        "tflops_exact_equivalent": achieved,
        "rechecked_points_per_step": rechecked,
        "resolved_in_kernel_per_step": resolved,
        "overflowed_per_step": overflowed,
        "fp64_check": check,
        "simt_fp32_step_ms": simt_s * 1e3 if simt_s is not None else None,
        "cpu_baseline": cpu, "gpu_launches": int(gpu_launches), "clocks": clocks,
    }


def _round_bf16(a):
    """float32 -> nearest bfloat16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _round_e4m3(a):
    """float64 values already scaled into e4m3's range -> nearest e4m3 value
    (3 mantissa bits, exponents -6..8, subnormal step 2^-9, max 448)."""
    a = np.asarray(a, np.float64)
    m, e = np.frexp(np.abs(a))                # |a| = m 2^e, m in [0.5, 1)
    step = np.ldexp(1.0, np.maximum(e - 4, -9))
    q = np.round(np.abs(a) / step) * step      # numpy rounds half to even
    return np.sign(a) * np.minimum(q, 448.0)


def precision_record(ckm, torch, dev, n, warm_iters=5, sample=4096):
    """Candidate fractions of the tensor-core certificate per operand
    precision, measured on the tensor-core workload (n points, d = 128,
    k = 1024, the 1024-component mixture) with the centroids after
    `warm_iters` real iterations of ckm_tc_fused_f32.  For each precision the
    sample's operands are rounded as the kernel would round them, the scores
    |c|^2 - 2 x.c are formed from the rounded operands, and the kernel's
    certificate T = t1 |x| + te |e| + t2 (|x| + cm)^2 (with fm, e the measured
    rounding-error norms of that precision) decides which clusters stay
    candidates.  fp8 e4m3 gets a scale per point row and per centroid row
    (at least as fine as per-tile scales); 'fp16 hi/lo' is the three-product
    split x_h c_h + x_h c_l + x_l c_h.  The reference's FP32 label must be a
    candidate in every case (soundness)."""
    d, k = 128, 1024
    P = torch.empty(n * d, dtype=torch.float32, device=dev)
    ckm.generate_mixture_ex(P, n, d, k, SEED, center=("normal", 0.0, 2.0), sigma=("loguniform", 0.25, 1.0),
                            dirichlet=True)
    tcp = ckm.TensorCorePoints(P, n, d)
    C = [P.view(d, n)[:, :k].reshape(-1).clone(), torch.empty(k * d, dtype=torch.float32, device=dev)]
    L = torch.empty(n, dtype=torch.int32, device=dev)
    M = torch.empty(k, dtype=torch.int32, device=dev)
    S = ckm.new_scratch(d, k, dev)
    stats = torch.zeros(2, dtype=torch.int32, device=dev)
    for i in range(warm_iters):
        ckm.tc_fused(P, tcp, C[i % 2], C[(i + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stats)
        if i == 0:
            tcp.sort(k)
    torch.cuda.synchronize()
    Cc = C[warm_iters % 2].cpu().numpy()                       # column-major k x d
    rng = np.random.default_rng(17)
    idx = np.sort(rng.choice(n, size=sample, replace=False))
    Xcm = np.ascontiguousarray(P.view(d, n)[:, torch.from_numpy(idx).to(dev)].cpu().numpy())
    del P, tcp
    torch.cuda.empty_cache()
    O = oracle_module()
    ref = O.label_f32(Xcm.reshape(-1), sample, d, k, Cc)
    X = Xcm.T.astype(np.float64)                               # sample x d
    Cr = Cc.reshape(d, k).T.astype(np.float64)                 # k x d
    valid = np.all(np.isfinite(Cr), axis=1)
    Cv = np.where(valid[:, None], Cr, 0.0)
    cn2 = np.where(valid, (Cv * Cv).sum(1).astype(np.float32).astype(np.float64), np.inf)
    xn = np.sqrt((X * X).sum(1))
    cm = float(np.sqrt((Cv * Cv).sum(1)).max())
    g = 2 * d * 2.0 ** -23
    t2 = 2 * 2.0 ** -23 + 2 * (d + 2) * 2.0 ** -24

    def pow2_scale(maxabs, top):
        return np.ldexp(1.0, np.floor(np.log2(top / maxabs)).astype(int))

    def rounded(kind):
        if kind == "fp16":
            sx = float(pow2_scale(np.abs(X).max(), 2.0 ** 15))
            sc = float(pow2_scale(np.abs(Cv).max(), 2.0 ** 15))
            return (X * sx).astype(np.float16).astype(np.float64) / sx, \
                   (Cv * sc).astype(np.float16).astype(np.float64) / sc, 0.0
        if kind == "bf16":
            return _round_bf16(X), _round_bf16(Cv), 0.0
        if kind == "fp8 e4m3":
            sx = pow2_scale(np.maximum(np.abs(X).max(1), 1e-30), 448.0)[:, None]
            sc = pow2_scale(np.maximum(np.abs(Cv).max(1), 1e-30), 448.0)[:, None]
            return _round_e4m3(X * sx) / sx, _round_e4m3(Cv * sc) / sc, 0.0
        # fp16 hi/lo: the x_l c_l product is dropped (|x_l||c_l| <= 2^-22 |x||c|)
        sx = float(pow2_scale(np.abs(X).max(), 2.0 ** 15))
        sc = float(pow2_scale(np.abs(Cv).max(), 2.0 ** 15))
        xh = (X * sx).astype(np.float16).astype(np.float64)
        ch = (Cv * sc).astype(np.float16).astype(np.float64)
        xl = (X * sx - xh).astype(np.float16).astype(np.float64)
        cl = (Cv * sc - ch).astype(np.float16).astype(np.float64)
        return (xh + xl) / sx, (ch + cl) / sc, 2.0 ** -21

    table = {}
    for kind, mma_cost in (("fp16", 1.0), ("bf16", 1.0), ("fp8 e4m3", 0.5), ("fp16 hi/lo", 3.0)):
        Xr, Cq, dropped = rounded(kind)
        e = np.sqrt(((Xr - X) ** 2).sum(1))
        fm = float(np.sqrt(((Cq - Cv) ** 2).sum(1))[valid].max())
        t1 = 4 * fm + 4 * g * (cm + fm)
        te = 4 * (cm + fm) + 4 * g * (cm + fm)
        T = t1 * xn + te * e + (t2 + 2 * dropped) * (xn + cm) ** 2
        scores = cn2[None, :] - 2.0 * (Xr @ Cq.T)
        m = scores.min(1)
        cand = scores <= (m + T)[:, None]
        counts = cand.sum(1)
        table[kind] = {"relative_mma_work": mma_cost, "median_T": float(np.median(T)),
                       "points_with_2plus_candidates": float(np.mean(counts >= 2)),
                       "mean_candidates": float(counts.mean()), "max_candidates": int(counts.max()),
                       "points_over_8_candidates": float(np.mean(counts > 8)),
                       "reference_label_always_a_candidate": bool(np.all(cand[np.arange(sample), ref]))}
    return {"metric": "candidate fraction", "unit": "fraction of points", "n_gpus": 1,
            "config": {"workload": "tensor_core_precision_table", "n": n, "d": d, "k": k,
                       "centroids": "after %d iterations of ckm_tc_fused_f32 from the first k points" % warm_iters,
                       "sample_points": sample},
            "precisions": table}


def run_precision_workload(args, ckm, torch, dev):
    print(json.dumps(precision_record(ckm, torch, dev, args.tc_points or (1 << 24))), flush=True)
    return 0


def run_tensor_core_workload(args, ckm, torch, dev):
    rec = tensor_core_record(ckm, torch, dev, args.tc_points or (1 << 24), args.steps, args.warmup,
                             simt_compare=not args.no_simt_compare, cpu_baseline=not args.no_cpu_baseline,
                             precision=args.tc_precision)
    print(json.dumps(rec), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + ["batched", "tensor_core", "serving", "buffered",
                                                                   "precision"])
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=2000.0, help="serving: small jobs per second")
    ap.add_argument("--serve-large-rate", type=float, default=0.5, help="serving: large jobs per second")
    ap.add_argument("--serve-pool", type=int, default=512, help="serving: distinct small-job payloads")
    ap.add_argument("--serve-plain-jobs", type=int, default=300)
    ap.add_argument("--serve-round", type=int, default=0, help="serving: batched iterations per round (0 = library default)")
    ap.add_argument("--jobs", type=int, default=4096, help="batched workload: number of jobs")
    ap.add_argument("--batch-d", type=int, default=0, help="batched workload: keep only jobs of this d")
    ap.add_argument("--batch-min-k", type=int, default=0, help="batched workload: keep only jobs with k >= this")
    ap.add_argument("--batch-max-k", type=int, default=0, help="batched workload: keep only jobs with k < this")
    ap.add_argument("--batch-max-jobs", type=int, default=0, help="batched workload: keep at most this many jobs")
    ap.add_argument("--no-plain", action="store_true",
                    help="batched workload: time the batched launches alone (no plain loop, no graph)")
    ap.add_argument("--tc-points", type=int, default=0, help="tensor_core workload: points (default 2^24)")
    ap.add_argument("--tc-precision", default="fp16", choices=["fp16", "bf16"],
                    help="tensor_core workload: operand type of the distance GEMM")
    ap.add_argument("--buffered-points", type=int, default=0, help="buffered workload: points (default 2^31)")
    ap.add_argument("--buffered-budget", type=int, default=0,
                    help="buffered workload: device budget in bytes (default a quarter of the point bytes, "
                         "at most 32 GiB)")
    ap.add_argument("--buffered-iterations", type=int, default=50, help="buffered workload: iterations per step")
    ap.add_argument("--no-simt-compare", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=9)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-spatial", action="store_true",
                    help="default workload: time the caller's point order only (no spatial sort, no box pruning)")
    ap.add_argument("--no-sub-records", action="store_true",
                    help="default workload: skip the bounded tensor_core / batched / serving records of the line")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the FP64 oracle checks of the line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    workload = args.workload

    if args.impl == "reference":
        return run_reference_arm(args, workload if workload in WORKLOADS else DEFAULT_WORKLOAD)

    if workload in ("batched", "tensor_core", "serving", "buffered", "precision"):
        import importlib

        import torch
        ckm = importlib.import_module("cl-kmeans_gb300")
        run = {"batched": run_batched_workload, "tensor_core": run_tensor_core_workload,
               "serving": run_serving_workload, "buffered": run_buffered_workload,
               "precision": run_precision_workload}[workload]
        return run(args, ckm, torch, torch.device("cuda", 0))

    import importlib

    import torch

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    ckm = importlib.import_module("cl-kmeans_gb300")
    ckm.lib()
    n, d, k, blobs, slo, shi, iters_cfg = WORKLOADS[workload]
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()

    # --- inputs resident in HBM (generated on the device) ---------------------
    P = torch.empty(n * d, dtype=torch.float32, device=dev)
    ckm.generate_mixture(P, n, d, blobs, SEED + rank, sigma=(slo, shi))
    C = [torch.empty(k * d, dtype=torch.float32, device=dev) for _ in range(2)]
    C[0].copy_(P.view(d, n)[:, :k].reshape(-1))   # first_x: C[f*k+c] = P[f*n+c]
    C0_host = C[0].cpu().numpy().copy()
    L = torch.empty(n, dtype=torch.int32, device=dev)
    M = torch.empty(k, dtype=torch.int32, device=dev)
    S = ckm.new_scratch(d, k, dev)
    torch.cuda.synchronize()

    def step(i):
        ckm.fused(P, C[i % 2], C[(i + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stream)

    def timed(step_fn, it0):
        """K steps bracketed by a barrier + synchronize, CUDA events on the
        launching stream around the whole region and around every launch."""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = ckm.launch_count()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(args.steps):
            evs[i][0].record(stream)
            step_fn(it0 + i)
            evs[i][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
        launches = ckm.launch_count() - launches0
        total_ms = t_start.elapsed_time(t_end)
        per_launch_ms = [a_.elapsed_time(b_) for a_, b_ in evs]
        total_ms = ranks_max_ms(total_ms, world)
        return total_ms, per_launch_ms, launches

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    # the caller's point order
    u_total_ms, u_per_launch, u_launches = timed(step, args.warmup)
    it_next = args.warmup + args.steps
    spatial = None
    if not args.no_spatial:
        # the same points in spatial (Z-) order, prepared once outside the
        # timed steps (ckm_spatial_sort_f32); the pruned kernel's labels are
        # the reference's on these points, and perm maps them back
        torch.cuda.synchronize()
        ts0 = time.perf_counter()
        Ps, perm = ckm.spatial_sort(P, n, d, stream)
        torch.cuda.synchronize()
        prepare_ms = (time.perf_counter() - ts0) * 1e3

        def step_sorted(i):
            ckm.fused_sorted(Ps, C[i % 2], C[(i + 1) % 2], L, M, S, n, d, k, ckm.MODE_FINALIZE, stream)

        for i in range(args.warmup):
            step_sorted(it_next + i)
        it_next += args.warmup
        total_ms, per_launch_ms, gpu_launches = timed(step_sorted, it_next)
        spatial = {"prepare_ms": prepare_ms, "call": "ckm_spatial_sort_f32 once, then ckm_fused_sorted_f32 per step"}
    else:
        total_ms, per_launch_ms, gpu_launches = u_total_ms, u_per_launch, u_launches
    clocks = sampler.stop()
    value = replica_throughput(n * args.steps, world, total_ms)
    avg_launch_s = statistics.mean(per_launch_ms) / 1e3
    unsorted = {"value": replica_throughput(n * args.steps, world, u_total_ms), "ms_per_step": u_total_ms / args.steps,
                "call": "ckm_fused_f32 on the points in generation order"}

    # --- roofline of the fused kernel --------------------------------------
    bytes_per_point = 4 * d + 4
    achieved = bytes_per_point * n / avg_launch_s / 1e9
    peak, peak_kind = measured_hbm_peak()
    tpp = profiled_traffic_per_point("dram_bytes_per_point" if args.no_spatial else "dram_bytes_per_point_spatial")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind,
                "traffic": (tpp * n) if tpp is not None else None,
                "algorithmic_bytes_per_launch": bytes_per_point * n}
    u_achieved = bytes_per_point * n / (statistics.mean(u_per_launch) / 1e3) / 1e9
    unsorted["roofline_frac"] = u_achieved / peak

    # --- e2e through the C ABI with pinned host buffers --------------------
    e2e = None
    if args.e2e_steps > 0:
        hostP = torch.empty(n * d, dtype=torch.float32, pin_memory=True)
        hostP.copy_(P)
        hp = hostP.numpy()
        hostC = torch.empty(k * d, dtype=torch.float32, pin_memory=True)
        hostL = torch.empty(n, dtype=torch.int32, pin_memory=True)
        hostM = torch.empty(k, dtype=torch.int32, pin_memory=True)
        cfg = ckm.RunConfig(b"single_stage", b"feature_sum", b"unroll_vector", b"part_local", b"feature_sum",
                            local, 0, 0)
        info = ckm.RunInfo()
        times, windows = [], []
        for _ in range(args.e2e_steps + 1):
            hostC.numpy()[:] = C0_host
            t0 = time.perf_counter()
            ckm.check(ckm.lib().ckm_kmeans_run_f32(ctypes.byref(cfg), iters_cfg, d, n, k, hp.ctypes.data,
                                                   hostC.data_ptr(), hostM.data_ptr(), hostL.data_ptr(),
                                                   ctypes.byref(info)), "ckm_kmeans_run_f32")
            times.append(time.perf_counter() - t0)
            windows.append(info.total_time_ns / 1e6)
        # the median call: the host link and the host's memory are shared with
        # the box's other GPUs, and a call now and then takes 2-4x longer
        e2e_t = statistics.median(times[1:])
        window_ms = info.total_time_ns / 1e6
        e2e = {"value": n * iters_cfg / e2e_t, "unit": "pts*iter/s",
               "h2d_bytes_per_step": int(info.h2d_bytes), "d2h_bytes_per_step": int(info.d2h_bytes),
               "iterations_per_step": iters_cfg, "ms_per_step": e2e_t * 1e3,
               "statistic": "median of %d calls after the first" % (len(times) - 1),
               "ms_per_step_mean": statistics.mean(times[1:]) * 1e3,
               "ms_per_call": [t * 1e3 for t in times],
               "window_ms_per_call": windows,
               "first_call": "allocates the device buffers from the stream-ordered pool; not in ms_per_step",
               "total_time_window_ms": window_ms,
               "window_roofline_frac": bytes_per_point * n * iters_cfg / (window_ms / 1e3) / 1e9 / peak,
               "window": "the reference's TotalTime window (kmeans_single_stage.hpp:89-160): the spatial sort "
                         "and all %d iterations; window_roofline_frac counts the reference's 20 B per "
                         "point-iteration, while the run's intermediate iterations on the sorted copy write no "
                         "labels (nothing reads them: the last iteration labels the caller's order)" % iters_cfg}
        if not args.no_fp64_check and rank == 0:
            # the call's result against the FP64 oracle: centroids against the
            # FP64 means of the returned labels, masses against their counts
            e2e["fp64_check"] = fp64_means_check(hp, n, d, k, hostL.numpy().view(np.uint32), hostC.numpy(),
                                                 hostM.numpy().view(np.uint32))
        # the link that bounds the copies inside e2e: pinned H2D, 64 MiB chunks
        link_best, _ = ckm.transfer_probe(64 << 20, repeat=16, pinned=True, to_device=True, device=local)
        e2e["h2d_link_gbs"] = link_best
        e2e["h2d_link_ms_per_step"] = info.h2d_bytes / (link_best * 1e9) * 1e3 if link_best > 0 else None
        del hostP

    # --- CPU baseline (oracle port, single thread, bounded sample) ---------
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        n_s, it_s = 1 << 22, iters_cfg
        Ps = np.ascontiguousarray(P.view(d, n)[:, :n_s].cpu().numpy()).reshape(-1)
        cpu = cpu_baseline_record(Ps, n_s, d, k, it_s, "first %d points of the workload" % n_s)

    subs = {}
    if rank == 0 and world == 1 and not args.no_sub_records:
        # configs 3, 4 and 5 as bounded records of the same line (each in its
        # own scope, device memory released between them)
        del P, L, M, S
        if not args.no_spatial:
            del Ps, perm
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        fp64 = not args.no_fp64_check
        for name, fn in (("tensor_core", lambda: tensor_core_record(ckm, torch, dev, 1 << 24, 3, 3, fp64=fp64)),
                         ("tensor_core_bf16", lambda: tensor_core_record(ckm, torch, dev, 1 << 24, 3, 3,
                                                                         simt_compare=False, cpu_baseline=False,
                                                                         fp64=fp64, precision="bf16")),
                         ("batched", lambda: batched_record(ckm, torch, dev, 4096, 3, 3, fp64=fp64)),
                         ("serving", lambda: serving_record(ckm, torch, dev, 10.0, 2000.0, 0.5, 512, 100, 0,
                                                            with_70pct=False, burst_rounds=2, fp64=fp64)),
                         # config 2b at its size (2^31 x 16 pinned on the host, 32 GiB device
                         # budget), 5 of its 50 iterations
                         ("buffered", lambda: buffered_record(ckm, torch, dev, 1 << 31, 0, 5, 1))):
            try:
                subs[name] = fn()
            except Exception as ex:  # report, keep the headline
                subs[name] = {"error": "%s: %s" % (type(ex).__name__, ex)}
            torch.cuda.synchronize()
            torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": "pts*iter/s", "value": value, "unit": "pts*iter/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian mixture generated on the device)",
            "config": {"workload": workload, "n": n, "d": d, "k": k, "blobs": blobs, "sigma": [slo, shi],
                       "seed": SEED, "init": "first_x",
                       "layout": "column-major" + ("" if args.no_spatial else
                                                  ", points in spatial order (sorted once before the timed steps)"),
                       "l2": "inputs (%.1f GiB) larger than L2, no flush" % (n * (d + 1) * 4 / 2 ** 30),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(gpu_launches),
            "clocks": clocks, "spatial_order": spatial, "caller_order": unsorted,
        }
        line.update(subs)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
