"""ozgb_dgemm_device_noalloc (the entry point that allocates no device memory)
against ozgb_dgemm_device on the same inputs, through the C ABI.

Both run the same plan and kernels (b = 7, triangular pair set, round to
nearest), so the bar is the one of the other parity tests: bit-identical
results.  Two different products in a row check that the shared scratch array,
which keeps the previous call's contents, does not leak into the next result.
"""
import ctypes

import numpy as np
import pytest

from conftest import HAVE_GPU


def _noalloc(L, dA, dB, dC, M, N, K, s, stream):
    return L.ozgb_dgemm_device_noalloc(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N, s, stream)


def test_noalloc_rejects_oversized_and_bad_arguments(ozlib):
    """Argument and size checks come before any device work (CPU-safe)."""
    L = ozlib.load()
    p = ctypes.c_void_p(16)
    assert L.ozgb_dgemm_device_noalloc(0, 4, 4, p, 4, p, 4, p, 4, 8, None) == 1
    assert L.ozgb_dgemm_device_noalloc(4, 4, 4, None, 4, p, 4, p, 4, 8, None) == 7
    assert L.ozgb_dgemm_device_noalloc(4, 4, 4, p, 4, p, 4, p, 4, 17, None) == 7
    # 4096^3 at s = 9 needs ~600 MB of slice planes: beyond the fixed 64 MiB
    assert L.ozgb_dgemm_device_noalloc(4096, 4096, 4096, p, 4096, p, 4096, p, 4096, 9, None) == 11


@pytest.mark.gpu
def test_noalloc_matches_device_entry_point(ozlib, oracle):
    if not HAVE_GPU:
        pytest.skip("no GPU")
    import torch
    L = ozlib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    cases = [((300, 200, 500), 9, 1.0), ((130, 70, 1000), 8, 4.0), ((1024, 1024, 1024), 15, 0.5)]
    for (M, N, K), s, phi in cases:
        A = oracle.gen_phi((M, K), M + 1, phi)
        B = oracle.gen_phi((K, N), N + 2, phi)
        dA = torch.from_numpy(A).to(dev)
        dB = torch.from_numpy(B).to(dev)
        got = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
        assert _noalloc(L, dA, dB, got, M, N, K, s, stream) == 0
        h = ozlib.Handle()
        h.set_slices(s)
        h.set_bins(s)
        want = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
        assert h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, want.data_ptr(), N, stream) == 0
        torch.cuda.synchronize()
        assert h.sync() == 0, h.last_error()
        h.close()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64)), (M, N, K, s)
        # and the result itself is the oracle's
        ref = oracle.dgemm(A, B, 7, s, s, 0)
        assert np.array_equal(g.view(np.uint64), ref.view(np.uint64))


@pytest.mark.gpu
def test_noalloc_padded_leading_dimensions_on_a_side_stream(ozlib, oracle):
    """Leading dimensions wider than the matrices (lda > K, ldb > N, ldc > N) and a
    fresh stream other than the current one: the exponent passes, the splits and
    the epilogue honour the strides, and the clears of the shared array run on
    that stream.  Two calls in a row, each bit-identical to ozgb_dgemm_device and
    to the oracle; the columns of C past N are left untouched."""
    if not HAVE_GPU:
        pytest.skip("no GPU")
    import torch
    L = ozlib.load()
    dev = torch.device("cuda", 0)
    side = torch.cuda.Stream(dev)
    M, N, K, s = 130, 70, 200, 9
    lda, ldb, ldc = K + 24, N + 10, N + 6
    for rep in range(2):
        A = oracle.gen_phi((M, K), 71 + rep, 1.0)
        B = oracle.gen_phi((K, N), 72 + rep, 1.0)
        Ap = np.full((M, lda), 3.0e300)
        Ap[:, :K] = A
        Bp = np.full((K, ldb), -7.0e200)
        Bp[:, :N] = B
        dA = torch.from_numpy(Ap).to(dev)
        dB = torch.from_numpy(Bp).to(dev)
        got = torch.full((M, ldc), 5.5, dtype=torch.float64, device=dev)
        want = torch.full((M, ldc), 5.5, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            assert L.ozgb_dgemm_device_noalloc(M, N, K, dA.data_ptr(), lda, dB.data_ptr(), ldb, got.data_ptr(), ldc,
                                               s, side.cuda_stream) == 0
        side.synchronize()
        h = ozlib.Handle()
        h.set_slices(s)
        h.set_bins(s)
        assert h.dgemm_device(M, N, K, dA.data_ptr(), lda, dB.data_ptr(), ldb, want.data_ptr(), ldc,
                              side.cuda_stream) == 0
        side.synchronize()
        assert h.sync() == 0, h.last_error()
        h.close()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert np.array_equal(g.view(np.uint64), w.view(np.uint64))
        assert np.all(g[:, N:] == 5.5)
        ref = oracle.dgemm(A, B, 7, s, s, 0)
        assert np.array_equal(g[:, :N].view(np.uint64), ref.view(np.uint64))
