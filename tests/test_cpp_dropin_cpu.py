"""The C++ drop-in surface: a program written against the reference's
strategy classes (abstract_kmeans.hpp:106-130 operator(), the setters of
kmeans_single_stage.hpp:174-198 and kmeans_three_stage.hpp:245-321, the four
configuration structs, the float/uint32 and double/uint64 instantiations of
bench.cpp:469-503) compiles against csrc/host and links against libckm.so.
Built and run on the CPU; the program makes no GPU call."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdint>
#include <memory>
#include <vector>

#include "binary_format.hpp"
#include "configuration.hpp"
#include "factories.hpp"
#include "kmeans_buffered.hpp"
#include "kmeans_single_stage.hpp"
#include "kmeans_three_stage.hpp"
#include "measurement.hpp"

template <typename P, typename L, typename M>
static int use(size_t iterations, size_t d, std::shared_ptr<const std::vector<P>> points,
               std::shared_ptr<std::vector<P>> centroids, std::shared_ptr<std::vector<M>> masses,
               std::shared_ptr<std::vector<L>> labels) {
    Clustering::FusedConfiguration fused;
    fused.strategy = "cluster_merge";
    Clustering::LabelingConfiguration labeling;
    Clustering::MassUpdateConfiguration mass;
    mass.strategy = "part_private";
    Clustering::CentroidUpdateConfiguration update;
    update.strategy = "feature_sum_pardim";

    Clustering::KmeansSingleStage<P, L, M> single;
    single.set_fused(fused);
    Clustering::KmeansThreeStage<P, L, M> three;
    three.set_labeler(labeling);
    three.set_mass_updater(mass);
    three.set_centroid_updater(update);
    Clustering::KmeansSingleStageBuffered<P, L, M> single_buffered;
    single_buffered.set_fused(fused);
    Clustering::KmeansThreeStageBuffered<P, L, M> three_buffered;
    three_buffered.set_labeler(labeling);
    three_buffered.set_mass_updater(mass);
    three_buffered.set_centroid_updater(update);

    Clustering::AbstractKmeans<P, L, M>* strategies[] = {&single, &three, &single_buffered, &three_buffered};
    int runs = 0;
    for (auto* s : strategies) {
        auto measurement = (*s)(iterations, d, points, centroids, masses, labels);  // abstract_kmeans.hpp:106
        runs += measurement != nullptr;
    }
    return runs;
}

int main(int argc, char**) {
    // never taken: the program only has to compile, link and load
    if (argc > 1000) {
        return use<float, uint32_t, uint32_t>(1, 4, nullptr, nullptr, nullptr, nullptr) +
               use<double, uint64_t, uint64_t>(1, 4, nullptr, nullptr, nullptr, nullptr);
    }
    return 0;
}
"""


def _cuda_home():
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def test_reference_style_program_compiles_links_and_loads(ckm, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    ckm.lib()  # the library is built
    lib_dir = os.path.join(ROOT, "cl-kmeans_gb300", "lib")
    cuda = _cuda_home()
    cuda_lib = next((p for p in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                 os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(p)), None)
    src = tmp_path / "user.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "user"
    cmd = [cxx, "-std=c++17", "-O0", "-Wall", str(src), "-o", str(exe),
           "-I", os.path.join(ROOT, "cl-kmeans_gb300", "csrc", "host"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), "-L", lib_dir, "-lckm", "-Wl,-rpath," + lib_dir]
    if cuda_lib:
        cmd += ["-L", cuda_lib, "-lcudart", "-Wl,-rpath," + cuda_lib]
    else:
        cmd += ["-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-4000:]
    r = subprocess.run([str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 0, r.stdout[-2000:]


def test_every_public_header_compiles_on_its_own():
    """Each C++ header of the drop-in surface includes what it uses, and the
    C ABI header is valid C (what cgo / other FFIs see)."""
    import glob
    cxx, cc = shutil.which("g++"), shutil.which("gcc")
    if cxx is None or cc is None:
        pytest.skip("no g++ / gcc")
    cuda_inc = os.path.join(_cuda_home(), "include")
    host = os.path.join(ROOT, "cl-kmeans_gb300", "csrc", "host")
    inc = os.path.join(ROOT, "include")
    for h in sorted(glob.glob(os.path.join(host, "*.hpp"))):
        r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-x", "c++", "-I", host, "-I", inc, "-I", cuda_inc, h],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
        assert r.returncode == 0, (h, r.stdout[-2000:])
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-x", "c", os.path.join(inc, "ckm.h")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert r.returncode == 0, r.stdout[-2000:]
