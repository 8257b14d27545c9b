"""The UMMA cost the planner assumes, measured on this GPU.

The planner (oz_plan.cpp) partitions the bins so as to minimise the number of
UMMAs per K step, on the measured fact that a cta_group::1 tcgen05.mma costs
about the same number of SM cycles whatever its N (up to 240), M (64 or 128) or
kind: a narrow UMMA is not cheaper than a wide one.  tests/perf/umma_cost.cu
issues long runs of UMMAs on every SM and reports cycles per instruction; this
test builds and runs it and holds the assumption to it.
"""
import os
import shutil
import subprocess

import pytest

from conftest import HAVE_GPU, ROOT

pytestmark = pytest.mark.gpu


def test_umma_cost_does_not_depend_on_n(tmp_path):
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
        if len(f) == 6:
            cost[(f[0], int(f[1]), int(f[2]), int(f[3]))] = float(f[4])
    print("\n" + r.stdout)
    c48, c240, c256 = cost[("bf16", 128, 48, 2)], cost[("bf16", 128, 240, 2)], cost[("bf16", 128, 256, 2)]
    assert abs(c48 - c240) <= 0.1 * c240          # N = 48 costs as much as N = 240
    assert c240 <= c256 <= 1.15 * c240            # N = 256 a little more
    assert abs(cost[("bf16", 64, 256, 1)] - cost[("bf16", 128, 240, 1)]) <= 0.1 * c240  # M = 64 no cheaper
    assert abs(cost[("e4m3", 128, 48, 1)] - c48) <= 0.1 * c48  # nor the e4m3 kind
