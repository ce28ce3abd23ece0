"""The lockstep batch form's host helpers (hpsim_gb300/csrc/lockstep.cuh),
compiled with g++ and run on the CPU: per-beam launch records chunked into
merged launches, and the block -> beam search of the merged kernels against
a linear scan (tests/lockstep_host.cpp)."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda_runtime.h")):
            return os.path.join(cand, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


def test_segment_chunks_and_block_search(tmp_path):
    gxx = shutil.which("g++")
    inc = cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "lockstep_host")
    src = os.path.join(ROOT, "tests", "lockstep_host.cpp")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "hpsim_gb300", "csrc"),
                        "-I", inc, src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
