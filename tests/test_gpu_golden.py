"""GPU tests against the committed golden fixtures (no oracle run needed) and of the
precision knob on the device.

Bar: exponents, int8 slices and results bit-identical to the fixture digests of
the 256 x 512 x 128 workload in both profiles; results of the reference-harness
inputs within the stated normwise bound of the exact products; the device's
slice choice identical to the host knob's on the same statistics.
"""
import json
import os

import numpy as np
import pytest

from golden import inputs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
H = inputs.sha256


def _dgemm(h, A, B, mode):
    M, K = A.shape
    N = B.shape[1]
    assert h.setup(M, N, K, mode) == 0, h.last_error()
    C = np.empty((M, N))
    assert h.dgemm(M, N, K, A, B, C) == 0, h.last_error()
    return C


@pytest.fixture(scope="module")
def uniform_256x512x128():
    doc = json.load(open(os.path.join(GOLDEN, "uniform_256x512x128.json")))
    A, B = inputs.uniform_256x512x128_inputs()
    assert H(A) == doc["A"] and H(B) == doc["B"]
    return doc, np.ascontiguousarray(A), np.ascontiguousarray(B)


@pytest.mark.parametrize("s", [8, 9])
def test_uniform_256x512x128_gb300_profile(gpu_handle, uniform_256x512x128, s):
    doc, A, B = uniform_256x512x128
    want = doc["profiles"]["b7_s%d_tri_rn" % s]
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(s)
    d = gpu_handle.dump(A, B, want_q=False)
    assert H(d["er"]) == doc["er"] and H(d["ec"]) == doc["ec"]
    assert H(d["a_slices"]) == want["a_slices"] and H(d["b_slices"]) == want["b_slices"]
    C = _dgemm(gpu_handle, A, B, 1)
    assert H(C) == want["C"]


@pytest.mark.parametrize("name,mode", [("ref_accurate_b3_d29", 0), ("ref_fast_b7_d8", 1)])
def test_uniform_256x512x128_reference_profile(gpu_handle, uniform_256x512x128, name, mode):
    """The reference's own tables and truncating decode: the slices and the final
    bits equal those of the reference's arithmetic (its compiled decode made the
    fixture)."""
    doc, A, B = uniform_256x512x128
    want = doc["profiles"][name]
    gpu_handle.set_profile(1)
    C = _dgemm(gpu_handle, A, B, mode)
    assert H(C) == want["C"]
    d = gpu_handle.dump(A, B, want_q=False)
    assert H(d["a_slices"]) == want["a_slices"] and H(d["b_slices"]) == want["b_slices"]


def test_uniform_256x512x128_against_mpfr(gpu_handle, uniform_256x512x128):
    _, A, B = uniform_256x512x128
    z = np.load(os.path.join(GOLDEN, "uniform_256x512x128_mpfr.npz"))
    gpu_handle.set_error_bound(1e-15)
    C = _dgemm(gpu_handle, A, B, 1)[z["rows"], z["cols"]]
    mp = z["mpfr"]
    assert np.linalg.norm(C - mp) / np.linalg.norm(mp) <= 1e-15


@pytest.mark.parametrize("fi", [0.5, 1.0, 2.0, 4.0])
@pytest.mark.parametrize("bound", [1e-8, 1e-11, 1e-13, 1e-15])
def test_harness_inputs_meet_requested_bound(gpu_handle, fi, bound):
    """Reference-harness inputs (test.cpp:219-237): the precision knob on the
    device picks s and the result meets the bound against the exact product."""
    z = np.load(os.path.join(GOLDEN, "harness.npz"))
    tag = "fi%g" % fi
    A, B, exact = z["A_" + tag], z["B_" + tag], z["exact_" + tag]
    gpu_handle.set_error_bound(bound)
    C = _dgemm(gpu_handle, np.ascontiguousarray(A), np.ascontiguousarray(B), 1)
    assert np.linalg.norm(C - exact) / np.linalg.norm(exact) <= bound


@pytest.mark.parametrize("phi", [0.5, 1.0, 4.0])
def test_device_knob_matches_host_knob(gpu_handle, oracle, ozlib, phi):
    M, N, K = 300, 260, 1500
    A = oracle.gen_phi((M, K), 31, phi)
    B = oracle.gen_phi((K, N), 32, phi)
    f = lambda x: ((x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int32)
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for any_set in (1, 0):
        gpu_handle.set_schedule_search(any_set)
        for bound in (1e-9, 1e-13, 1e-15):
            s_host, J_host, _ = ozlib.choose_schedule(f(A).max(axis=1), (A * A).sum(axis=1), f(B).max(axis=0),
                                                      (B * B).sum(axis=0), K, 7, bound, (A * A).sum(axis=0),
                                                      (B * B).sum(axis=1), any_pair_set=any_set, sms=sms)
            gpu_handle.set_error_bound(bound)
            C = _dgemm(gpu_handle, A, B, 1)
            cfg = gpu_handle.config()
            assert (cfg["slices"], cfg["bins"]) == (s_host, J_host)
            ref = oracle.dgemm(A, B, 7, s_host, J_host, 0)
            assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("phi", [1.0, 4.0])
def test_device_elementwise_knob_matches_host_knob(gpu_handle, oracle, ozlib, phi):
    """The elementwise criterion on the device (flattest row and column from the
    stage-(a) partial sums) picks the host knob's slice count."""
    M, N, K = 300, 260, 1500
    A = oracle.gen_phi((M, K), 33, phi)
    B = oracle.gen_phi((K, N), 34, phi)
    f = lambda x: ((x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int32)
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    gpu_handle.set_error_criterion(ozlib.Criterion.elementwise, 1e-3)
    for bound in (1e-9, 1e-13):
        s_host, J_host, _ = ozlib.choose_schedule(f(A).max(axis=1), (A * A).sum(axis=1), f(B).max(axis=0),
                                                  (B * B).sum(axis=0), K, 7, bound, (A * A).sum(axis=0),
                                                  (B * B).sum(axis=1), criterion=1, tail=1e-3, sms=sms)
        gpu_handle.set_error_bound(bound)
        C = _dgemm(gpu_handle, A, B, 1)
        cfg = gpu_handle.config()
        assert (cfg["slices"], cfg["bins"]) == (s_host, J_host)
        ref = oracle.dgemm(A, B, 7, s_host, J_host, 0)
        assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
