"""Builds libckm.so (CUDA kernels for sm_103a + the C ABI + the C++ strategy
layer) and the ckm_bench command-line tool, in-tree.

    python cl-kmeans_gb300/build.py [--force] [-j N]

Objects go to cl-kmeans_gb300/_build/, the library to
cl-kmeans_gb300/lib/libckm.so, the tool to cl-kmeans_gb300/bin/ckm_bench.
A target is rebuilt when any of its sources or any header is newer.
"""
import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libckm.so")
BENCH_BIN = os.path.join(BINDIR, "ckm_bench")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp"))) + sorted(
        f for f in glob.glob(os.path.join(CSRC, "host", "*.cpp")) if not f.endswith("bench_main.cpp"))
    return cu, cpp


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.hpp"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _obj(src):
    rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
    return os.path.join(BUILD, rel + ".o")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force=False, jobs=None, verbose=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    cu, cpp = _sources()
    hdr_time = _newest(_headers())
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    cmds = []
    for s in cu:
        o = _obj(s)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            cmds.append([nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", "-Xptxas", "-v" if verbose else "-O3"] + inc + ["-c", s, "-o", o])
    for s in cpp:
        o = _obj(s)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"] + inc +
                        ["-c", s, "-o", o])
    jobs = jobs or min(16, os.cpu_count() or 4)
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            outs = list(ex.map(_run, cmds))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    objs = [_obj(s) for s in cu + cpp]
    if force or cmds or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lpthread"])
    bench_src = os.path.join(CSRC, "host", "bench_main.cpp")
    if os.path.exists(bench_src):
        if force or not os.path.exists(BENCH_BIN) or os.path.getmtime(BENCH_BIN) < max(
                os.path.getmtime(bench_src), os.path.getmtime(LIB), hdr_time):
            _run(["g++", "-O3", "-std=c++17"] + inc + [bench_src, "-o", BENCH_BIN, "-L" + LIBDIR, "-lckm",
                  "-Wl,-rpath,$ORIGIN/../lib", "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-lpthread"])
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.j, verbose=a.verbose))
    sys.exit(0)
