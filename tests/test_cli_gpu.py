"""ckm_bench end to end (the reference's bench workflow, bench.cpp:201-450):
.conf + binary feature file in, --verify against the KmeansNaive arithmetic,
and the three CSV files of Measurement::write_csv (measurement.cpp:203-324)."""
import csv
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import blobs
from test_cli_cpu import bench_bin

pytestmark = pytest.mark.gpu

CONF = """
[benchmark]
runs = {runs}
verify = false
[kmeans]
clusters = {k}
pipeline = {pipeline}
iterations = {iters}
converge = false
types.point = {pt}
types.label = {lt}
types.mass = {lt}
[kmeans.labeling]
strategy = unroll_vector
global_size = 32768
local_size = 64
vector_length = 2
[kmeans.mass_update]
strategy = part_private
global_size = 32768
local_size = 32
vector_length = 4
[kmeans.centroid_update]
strategy = feature_sum_pardim
global_size = 32768
local_size = 64
local_features = 4
vector_length = 4
[kmeans.fused]
strategy = feature_sum
global_size = 32768
local_size = 32
vector_length = 4
[kmeans.gb300]
chunk_mib = 1
"""


def write_points(path, n, d, seed):
    P = blobs(n, d, 8, seed=seed)
    with open(path, "wb") as fh:
        np.array([d, 0, n], np.uint64).tofile(fh)
        P.tofile(fh)
    return P


@pytest.mark.parametrize("pipeline", ["single_stage", "three_stage", "single_stage_buffered",
                                      "three_stage_buffered"])
@pytest.mark.parametrize("types", [("float", "uint32"), ("double", "uint64")])
def test_bench_verify(ckm, cuda, tmp_path, pipeline, types):
    n, d, k = 200003, 4, 8     # 200003 * 4 * 4 B = 3.05 MiB -> 4 chunks of 1 MiB when buffered
    data = tmp_path / "points.bin"
    write_points(data, n, d, seed=5)
    conf = tmp_path / "run.conf"
    conf.write_text(CONF.format(runs=1, k=k, pipeline=pipeline, iters=10, pt=types[0], lt=types[1]))
    r = subprocess.run([bench_bin(ckm), "--config", str(conf), "--verify", str(data)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    mism = int(fields[fields.index("labels_mismatch") + 1])
    mse = float(fields[fields.index("centroid_mse") + 1])
    assert mism <= 2, r.stdout          # near-ties only (FP64-merged vs Kahan FP32 centroids)
    assert mse < 1e-10, r.stdout


def test_bench_csv_files(ckm, cuda, tmp_path):
    n, d, k = 50000, 3, 6
    data = tmp_path / "set.bin"
    write_points(data, n, d, seed=6)
    conf = tmp_path / "run.conf"
    conf.write_text(CONF.format(runs=2, k=k, pipeline="single_stage", iters=7, pt="float", lt="uint32"))
    out = tmp_path / "csv"
    out.mkdir()
    r = subprocess.run([bench_bin(ckm), "--config", str(conf), "--csv", str(out / "res.csv"), "--verbose",
                        str(data)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "2 runs, in" in r.stdout
    expm = sorted(glob.glob(str(out / "*_res_expm.csv")))
    mnts = sorted(glob.glob(str(out / "*_res_mnts.csv")))
    evnt = sorted(glob.glob(str(out / "*_res_evnt.csv")))
    assert len(expm) == len(mnts) == len(evnt) == 2
    rows = list(csv.reader(open(expm[0])))
    assert rows[0] == ["ExperimentID", "ParameterName", "Value"]
    params = {r[1]: r[2] for r in rows[1:]}
    for key in ("NumFeatures", "NumPoints", "NumClusters", "Filename", "Hostname", "Version", "TimeStamp",
                "FusedGlobalSize", "FusedLocalSize", "FusedVectorLength"):
        assert key in params, key
    assert params["NumPoints"] == str(n) and params["NumClusters"] == str(k) and params["Filename"] == "set.bin"
    rows = list(csv.reader(open(mnts[0])))
    assert rows[0] == ["ExperimentID", "Run", "TypeName", "Iteration", "Value"]
    names = [r[2] for r in rows[1:]]
    assert names.count("FusedFeatureSum") == 7 and "TotalTime" in names and "PointsH2D" in names
    rows = list(csv.reader(open(evnt[0])))
    assert rows[0] == ["ExperimentID", "Run", "TypeName", "Iteration", "CommandQueueID", "Queued", "Submit",
                       "Start", "End"]
    for r in rows[1:]:
        assert int(r[8]) >= int(r[7]) > 0


def test_generate_then_read(ckm, cuda, tmp_path):
    f = tmp_path / "gen.bin"
    r = subprocess.run([bench_bin(ckm), "--generate", str(f), "--points", "10000", "--features", "5",
                        "--blobs", "7", "--seed", "9"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    hdr = np.fromfile(f, np.uint64, 3)
    assert list(hdr) == [5, 0, 10000]
    body = np.fromfile(f, np.float32, offset=24)
    assert body.size == 50000 and np.isfinite(body).all()


def test_transfer_probe(ckm, cuda):
    """ckm_transfer_probe: positive, plausible link throughputs in both
    directions for pinned and pageable host memory."""
    best, mean = ckm.transfer_probe(16 << 20, repeat=8, pinned=True, to_device=True)
    assert 1.0 < best < 2000.0 and 0.0 < mean <= best * (1 + 1e-9)
    for pinned, to_device in ((True, False), (False, True), (False, False)):
        b, m = ckm.transfer_probe(4 << 20, repeat=4, pinned=pinned, to_device=to_device)
        assert b > 0.0 and m > 0.0


def test_bench_transfer_mode(ckm, cuda):
    """ckm_bench --transfer (the reference's transfer_bench measurement):
    one CSV line per chunk size, direction and host memory kind."""
    import subprocess
    r = subprocess.run([ckm.BENCH_BIN, "--transfer", "--max-size", "4", "--repeat", "4"], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0] == "direction,host_memory,chunk_mib,repeat,best_gbs,mean_gbs"
    rows = [l.split(",") for l in lines[1:]]
    assert len(rows) == 3 * 4   # 1, 2, 4 MiB x {H2D, D2H} x {pinned, pageable}
    assert {r[0] for r in rows} == {"H2D", "D2H"} and {r[1] for r in rows} == {"pinned", "pageable"}
    assert all(float(r[4]) > 0 for r in rows)
