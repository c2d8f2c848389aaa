"""Build libmkf_gb300.so (sm_103a) in-tree with nvcc: one object per .cu,
compiled in parallel, linked with the static CUDA runtime."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmkf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"] + ARCH


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(HERE, "..", "include", "mkf_gb300.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(HERE, "..", "include", "mkf_gb300.h")]
    jobs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [nv] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", src, "-o", obj]
            jobs.append((src, cmd))
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in sources()]

    def run(job):
        src, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for src, r in ex.map(run, jobs):
                if verbose or ptxas_v or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError("nvcc failed on %s" % src)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nv, "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libmkf_gb300.so failed")
        os.replace(tmp, LIB)
    return LIB


HARNESS_DIR = os.path.join(HERE, "harness")
HARNESS = os.path.join(HARNESS_DIR, "mkf_harness")
INCLUDE = os.path.join(HERE, "..", "include")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def build_harness(force: bool = False) -> str:
    """The standalone C++ harness (host code only, g++), linked against
    libmkf_gb300.so (found next to the package through its rpath) and the
    static CUDA runtime."""
    lib = build()
    src = os.path.join(HARNESS_DIR, "mkf_harness.cpp")
    deps = [src, lib, os.path.join(HARNESS_DIR, "mkf_yaml.hpp"), os.path.join(INCLUDE, "mkf_gb300.hpp"),
            os.path.join(INCLUDE, "mkf_gb300.h")]
    if not force and not _stale(HARNESS, deps):
        return HARNESS
    cxx = shutil.which("g++") or "g++"
    cuda = cuda_home()
    tmp = HARNESS + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, "-I", os.path.join(cuda, "include"), src, "-o", tmp,
           "-L", HERE, "-lmkf_gb300", "-Wl,-rpath,$ORIGIN/..", "-L", os.path.join(cuda, "lib64"),
           "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("g++ failed on the harness")
    os.replace(tmp, HARNESS)
    return HARNESS


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv))
    print(build_harness(force="--force" in sys.argv))
