"""The UMMA cost the planner assumes, measured on this GPU.

The planner (oz_plan.cpp) partitions the bins so as to minimise the number of
UMMAs per K step, on the measured fact that a cta_group::1 tcgen05.mma costs
about the same number of SM cycles whatever its N up to about 200, its M (64 or
128) or its kind, and only a little more at N = 256: a narrow UMMA is not cheaper
than a wide one.  tests/perf/umma_cost.cu
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
    c16, c48, c128, c192 = (cost[("bf16", 128, n, 2)] for n in (16, 48, 128, 192))
    c256 = cost[("bf16", 128, 256, 2)]
    # a narrow UMMA is not cheaper than a 192-wide one ...
    assert max(c16, c48, c128) >= 0.9 * c192
    # ... and the widest costs far less than twice a 128-wide one
    assert c256 <= 1.3 * c128
    # M = 64 is no cheaper than M = 128, nor the e4m3 kind than bf16, at the same N
    assert cost[("bf16", 64, 128, 2)] >= 0.9 * c128
    assert abs(cost[("e4m3", 128, 48, 1)] - cost[("bf16", 128, 48, 1)]) <= 0.1 * c48
