"""The UMMA costs the slice-pair GEMM's planner assumes, measured on this GPU.

The planner (oz_plan.cpp) and the kernel's issuing scheme rest on three measured
facts about cta_group::1 tcgen05.mma (M = 128, K = 16, bf16) on GB300:

* the tensor pipe takes about N / 2 SM cycles for a UMMA of N columns (the
  widest, N = 256, in about 128);
* one issuing thread issues a UMMA no faster than about every 70-110 cycles, so
  narrow UMMAs from one thread leave the pipe idle;
* a second issuing warp on another scheduler raises the rate of narrow UMMAs
  (the kernel deals each K step's UMMA runs to up to three issuing warps).

tests/perf/umma_cost.cu measures them on every SM; this test builds and runs it
and holds the assumptions to it.
"""
import os
import shutil
import subprocess

import pytest

from conftest import HAVE_GPU, ROOT

pytestmark = pytest.mark.gpu


def test_umma_cost_model(tmp_path):
    if not HAVE_GPU:
        pytest.skip("no GPU")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    nvcc = nvcc if os.path.exists(nvcc) else shutil.which("nvcc")
    exe = str(tmp_path / "umma_cost")
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", exe,
                           os.path.join(ROOT, "tests", "perf", "umma_cost.cu")])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    cost = {}
    for line in r.stdout.split("\n"):
        f = line.split()
        if len(f) == 4:
            cost[(f[0], int(f[1]), int(f[2]))] = float(f[3])
    print("\n" + r.stdout)
    tight = {n: cost[("tight", n, 1)] for n in (16, 48, 96, 128, 192, 256)}
    # wide UMMAs: half a cycle per column
    assert 0.45 * 256 <= tight[256] <= 0.6 * 256
    assert 0.45 * 192 <= tight[192] <= 0.65 * 192
    # narrow UMMAs: the issuing thread's floor, the same for every narrow N
    floor = tight[16]
    assert 50 <= floor <= 130
    assert abs(tight[48] - floor) <= 0.1 * floor
    # a second issuing warp raises the rate of narrow UMMAs by at least a third
    assert cost[("pairs", 48, 2)] <= 0.75 * cost[("pairs", 48, 1)]
