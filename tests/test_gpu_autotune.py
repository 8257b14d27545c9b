"""The autotuner on the GPU: it records a feasible plan for the size class, later
calls use it, and the results do not depend on the plan (the accumulation is
exact, so every plan rounds the same integer).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_changes_plan_not_results(gpu_handle, oracle, ozlib):
    from ozaie_gb300 import api
    api.tuning_clear()
    M, N, K = 640, 528, 1024
    A = oracle.gen_phi((M, K), 61, 1.0)
    B = oracle.gen_phi((K, N), 62, 1.0)
    gpu_handle.set_slices(9)
    gpu_handle.set_bins(9)
    assert gpu_handle.setup(M, N, K, 1) == 0
    before = np.empty((M, N))
    assert gpu_handle.dgemm(M, N, K, A, B, before) == 0, gpu_handle.last_error()
    untuned = gpu_handle.config()
    best = gpu_handle.autotune(M, N, K, 7, 9, 9, max_candidates=12)
    assert api.tuning_entries() == 1
    assert (best["slices"], best["bins"]) == (9, 9)
    after = np.empty((M, N))
    assert gpu_handle.dgemm(M, N, K, A, B, after) == 0, gpu_handle.last_error()
    tuned = gpu_handle.config()
    for key in ("tile_n", "k_chunk", "stages", "blocks", "block_lo", "block_nb"):
        assert tuned[key] == best[key], key
    assert np.array_equal(before.view(np.uint64), after.view(np.uint64))
    ref = oracle.dgemm(A, B, 7, 9, 9, 0)
    assert np.array_equal(after.view(np.uint64), ref.view(np.uint64))
    api.tuning_clear()
    assert api.tuning_entries() == 0
    assert untuned["slices"] == 9
