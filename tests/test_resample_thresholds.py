"""The exact resampler's 64-bit threshold arithmetic (shared by every GPU
resampling kernel) against the 128-bit rule it restates, compiled for the host
from the kernels' own header."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None


def test_rs_threshold_matches_128_bit_rule(tmp_path):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "rs_threshold_check")
    src = os.path.join(ROOT, "tests", "rs_threshold_check.cpp")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "mkfbodytracker_pdaf_gb300", "csrc"),
                    "-I", inc, src, "-o", exe], check=True)
    bad, n = map(int, subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split())
    assert n > 400000
    assert bad == 0, "%d of %d thresholds differ from the 128-bit rule" % (bad, n)
