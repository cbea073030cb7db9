"""The bench front-end's host logic without a GPU: the .conf parser (keys of
configuration_parser.cpp:43-111, 1-3 element size lists padded with 1 as in
:174-191, unknown keys rejected like Boost program_options), and the binary
feature-file header (binary_format.cpp:20-46)."""
import os
import subprocess

import numpy as np
import pytest


def bench_bin(ckm):
    if not os.path.exists(ckm.BENCH_BIN):
        ckm.build()
    return ckm.BENCH_BIN


def parse(ckm, tmp_path, text):
    p = tmp_path / "x.conf"
    p.write_text(text)
    r = subprocess.run([bench_bin(ckm), "--config", str(p), "--print-config"], capture_output=True, text=True)
    if r.returncode != 0:
        raise ValueError(r.stderr.strip())
    return dict(line.split("=", 1) for line in r.stdout.strip().splitlines())


THREE_STAGE = """
[benchmark]
runs = 3
verify = true

[kmeans]
clusters = 12
pipeline = three_stage   # inline comment
iterations = 25
converge = false
types.point = float
types.label = uint32
types.mass = uint32

[kmeans.labeling]
platform = 0
device = 0
strategy = unroll_vector
global_size = 8192
local_size = 128
vector_length = 2
unroll_clusters_length = 4
unroll_features_length = 2

[kmeans.mass_update]
platform = 0
device = 0
strategy = part_global
global_size = 1024 2
local_size = 64
vector_length = 8

[kmeans.centroid_update]
platform = 0
device = 0
strategy = cluster_merge
global_size = 4096, 3, 2
local_size = 32
local_features = 2
thread_features = 1
vector_length = 1
"""


def test_three_stage_conf(ckm, tmp_path):
    c = parse(ckm, tmp_path, THREE_STAGE)
    assert c["benchmark.runs"] == "3" and c["benchmark.verify"] == "1"
    assert c["kmeans.clusters"] == "12" and c["kmeans.pipeline"] == "three_stage"
    assert c["kmeans.iterations"] == "25"
    assert c["kmeans.labeling.global_size"] == "8192,1,1"      # padded with 1
    assert c["kmeans.mass_update.global_size"] == "1024,2,1"
    assert c["kmeans.centroid_update.global_size"] == "4096,3,2"
    assert c["kmeans.mass_update.strategy"] == "part_global"
    assert c["kmeans.centroid_update.strategy"] == "cluster_merge"
    assert c["kmeans.labeling.unroll_clusters_length"] == "4"
    # unset sections keep their defaults
    assert c["kmeans.fused.strategy"] == "feature_sum"


def test_fused_conf_and_gb300_section(ckm, tmp_path):
    c = parse(ckm, tmp_path, """
[kmeans]
clusters = 16
pipeline = single_stage_buffered
iterations = 50
types.point = double
types.label = uint64
types.mass = uint64
[kmeans.fused]
strategy = cluster_merge
global_size = 32768
local_size = 32
vector_length = 4
[kmeans.gb300]
device_budget_mib = 32768
chunk_mib = 512
""")
    assert c["kmeans.types.point"] == "double" and c["kmeans.types.label"] == "uint64"
    assert c["kmeans.fused.strategy"] == "cluster_merge" and c["kmeans.fused.vector_length"] == "4"
    assert c["kmeans.gb300.device_budget_mib"] == "32768" and c["kmeans.gb300.chunk_mib"] == "512"


@pytest.mark.parametrize("bad, msg", [
    ("[kmeans]\nclustres = 4\n", "unrecognised option"),
    ("[kmeans]\nclusters = four\n", "invalid value"),
    ("[kmeans]\nclusters = -3\n", "invalid value"),
    ("[benchmark]\nverify = maybe\n", "invalid value"),
    ("[kmeans.fused]\nglobal_size = 1 2 3 4\n", "more than 3"),
    ("[kmeans]\nclusters = 4\nclusters = 5\n", "more than once"),
    ("[kmeans\nclusters = 4\n", "bad section"),
])
def test_bad_conf_is_rejected(ckm, tmp_path, bad, msg):
    with pytest.raises(ValueError) as e:
        parse(ckm, tmp_path, bad)
    assert msg in str(e.value)


def test_binary_header(ckm, tmp_path):
    n, d = 1234, 7
    f = tmp_path / "p.bin"
    with open(f, "wb") as fh:
        np.array([d, 0, n], np.uint64).tofile(fh)
        np.zeros(n * d, np.float32).tofile(fh)
    r = subprocess.run([bench_bin(ckm), "--info", str(f)], capture_output=True, text=True)
    assert r.returncode == 0
    info = dict(line.split("=") for line in r.stdout.split())
    assert info == {"num_features": "7", "num_clusters": "0", "num_points": "1234"}
    r = subprocess.run([bench_bin(ckm), "--info", str(tmp_path / "missing.bin")], capture_output=True, text=True)
    assert r.returncode != 0 and "cannot open" in r.stderr


def test_converge_and_tolerance_keys(ckm, tmp_path):
    """kmeans.converge (parsed but unused in the reference,
    configuration_parser.cpp:67, 143-145) drives the convergence test here;
    its tolerance is [kmeans.gb300] tolerance, a positive real (default 1e-4)."""
    base = "[kmeans]\nclusters = 4\npipeline = single_stage\niterations = 50\nconverge = true\n"
    c = parse(ckm, tmp_path, base)
    assert c["kmeans.converge"] == "1" and float(c["kmeans.gb300.tolerance"]) == 1e-4
    c = parse(ckm, tmp_path, base + "[kmeans.gb300]\ntolerance = 2.5e-3\n")
    assert float(c["kmeans.gb300.tolerance"]) == 2.5e-3
    for bad in ("0", "-1e-3", "abc"):
        with pytest.raises(ValueError):
            parse(ckm, tmp_path, base + "[kmeans.gb300]\ntolerance = %s\n" % bad)


def test_spatial_order_key(ckm, tmp_path):
    """[kmeans.gb300] spatial_order = auto | on | off (default auto)."""
    base = "[kmeans]\nclusters = 4\npipeline = single_stage\niterations = 10\n"
    assert parse(ckm, tmp_path, base)["kmeans.gb300.spatial_order"] == "auto"
    for v in ("on", "off", "auto"):
        c = parse(ckm, tmp_path, base + "[kmeans.gb300]\nspatial_order = %s\n" % v)
        assert c["kmeans.gb300.spatial_order"] == v
    with pytest.raises(ValueError):
        parse(ckm, tmp_path, base + "[kmeans.gb300]\nspatial_order = sometimes\n")
