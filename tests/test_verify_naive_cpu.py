"""The CPU reference of `ckm_bench --verify` (csrc/host/verify_naive.hpp, a
restatement of the reference's KmeansNaive, kmeans_naive.cpp:40-103) pinned
bit-for-bit to the golden fixtures the reference itself produced
(tests/golden/*.npz): labels, masses and centroids, NaN positions included.
A small driver compiles the header as ckm_bench does (g++ -O3) and runs each
fixture's points from its initial centroids for its iteration count."""
import glob
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "verify_naive.hpp"

template <typename P, typename I>
int run(const char* dir, size_t n, size_t d, size_t k, unsigned iters) {
    std::vector<P> pts(n * d), C(k * d);
    std::vector<I> masses(k), labels(n);
    auto rd = [&](const char* name, void* dst, size_t bytes) {
        char path[4096];
        std::snprintf(path, sizeof(path), "%s/%s", dir, name);
        FILE* f = std::fopen(path, "rb");
        if (!f || std::fread(dst, 1, bytes, f) != bytes) std::exit(2);
        std::fclose(f);
    };
    auto wr = [&](const char* name, const void* src, size_t bytes) {
        char path[4096];
        std::snprintf(path, sizeof(path), "%s/%s", dir, name);
        FILE* f = std::fopen(path, "wb");
        if (!f || std::fwrite(src, 1, bytes, f) != bytes) std::exit(3);
        std::fclose(f);
    };
    rd("points.bin", pts.data(), pts.size() * sizeof(P));
    rd("c0.bin", C.data(), C.size() * sizeof(P));
    verify_naive<P, I, I>(iters, pts, n, d, C, masses, labels);
    wr("c.bin", C.data(), C.size() * sizeof(P));
    wr("m.bin", masses.data(), masses.size() * sizeof(I));
    wr("l.bin", labels.data(), labels.size() * sizeof(I));
    return 0;
}

int main(int argc, char** argv) {
    const size_t n = std::strtoull(argv[2], 0, 10), d = std::strtoull(argv[3], 0, 10),
                 k = std::strtoull(argv[4], 0, 10);
    const unsigned it = (unsigned)std::strtoul(argv[5], 0, 10);
    if (argv[6][0] == '3') return run<float, unsigned int>(argv[1], n, d, k, it);
    return run<double, unsigned long long>(argv[1], n, d, k, it);
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("verify_naive")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    subprocess.run(["g++", "-O3", "-std=c++17", "-I", os.path.join(ROOT, "cl-kmeans_gb300", "csrc", "host"),
                    str(src), "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_verify_reference_reproduces_reference_golden(driver, tmp_path, path):
    z = np.load(path)
    n, d, k, it = [int(x) for x in z["shape"]]
    f32 = str(z["type"]) == "f32"
    z["points"].tofile(tmp_path / "points.bin")
    z["centroids0"].tofile(tmp_path / "c0.bin")
    subprocess.run([driver, str(tmp_path), str(n), str(d), str(k), str(it), "32" if f32 else "64"], check=True)
    ft, it_ = (np.float32, np.uint32) if f32 else (np.float64, np.uint64)
    C = np.fromfile(tmp_path / "c.bin", ft)
    M = np.fromfile(tmp_path / "m.bin", it_)
    L = np.fromfile(tmp_path / "l.bin", it_)
    bits = np.uint32 if f32 else np.uint64
    assert np.array_equal(L, z["labels"].astype(it_))
    assert np.array_equal(M, z["masses"].astype(it_))
    assert np.array_equal(C.view(bits), np.asarray(z["centroids"], ft).view(bits))
