"""The integer paths that the GPU particle kernels share (Philox4x32-10; the
exact resampler's scatter walk, 128-bit search, 64-bit thresholds, weight
quantisation by bit fields and interleaved branch-free search; the
table-driven component pick), compiled for
the host from the kernels' own header and checked against independent
restatements (tests/integer_paths_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("ip") / "integer_paths_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "mkfbodytracker_pdaf_gb300", "csrc"),
                    "-I", inc, os.path.join(ROOT, "tests", "integer_paths_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {name: (int(bad), int(n)) for name, bad, n in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("piece,min_cases", [("thresholds", 400000), ("stride", 100000), ("quantize", 1000000), ("search", 400000),
                                             ("pick", 6000000), ("pickbin", 16777216), ("philox", 3), ("philox_split", 1000000),
                                             ("walk", 1000000)])
def test_against_independent_restatement(results, piece, min_cases):
    bad, n = results[piece]
    assert n >= min_cases
    assert bad == 0, "%s: %d of %d cases differ" % (piece, bad, n)
