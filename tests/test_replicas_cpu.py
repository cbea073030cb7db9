"""bench.py --gpus N: N independent replicas (the Lloyd iteration is run
whole on every rank; no data-path collective).  The host side is a gloo
process group: a barrier before the timed region, the slowest rank's time by
an all-reduce MAX, and whole-job throughput = all ranks' units over that
time; the reference arm runs on rank 0 only.  Checked here with two gloo
ranks on the CPU (no GPU)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        mine = 100.0 + 25.0 * rank          # this rank's timed region (ms)
        worst = bench.ranks_max_ms(mine, world)
        value = bench.replica_throughput(1000, world, worst)

        class Args:  # the reference arm's early exit on ranks other than 0
            steps = 1
            warmup = 0
        ref_rc = bench.run_reference_arm(Args(), bench.DEFAULT_WORKLOAD) if rank != 0 else None
        out.put((rank, worst, value, ref_rc))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_the_whole_job_throughput():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(out.get(timeout=5) for _ in range(2))
    for rank, worst, value, ref_rc in got:
        assert worst == pytest.approx(125.0)                    # max over the two ranks
        assert value == pytest.approx(2 * 1000 / 0.125)          # 2 ranks x 1000 units in 125 ms
    assert got[1][3] == 0                                        # rank 1 skips the reference arm


def test_single_rank_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.ranks_max_ms(42.0, 1) == 42.0
    assert bench.replica_throughput(500, 1, 250.0) == pytest.approx(2000.0)


def test_reference_arm_line_on_the_cpu():
    """bench.py --impl reference times the reference's CPU path (its own
    KmeansNaive32 compiled unchanged into oracle/_ref, single-threaded; the
    oracle port only where that build is absent) and prints one JSON line with
    the contract's keys; it needs no GPU."""
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "pts*iter/s" and line["unit"] == "pts*iter/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["warmup"] >= 3
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["sample"]
    import oracle as O
    if O.ref_available():
        assert cpu["kind"] == "reference" and cpu["cores"] == 1
    assert line["port_threaded"]["cores"] >= 1 and line["port_threaded"]["value"] > 0
    assert cpu["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == "lloyd_n2^28_d4_k16"
