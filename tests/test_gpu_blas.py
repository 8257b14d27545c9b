"""The BLAS-style entry point (ozgb_dgemm_ex) on the GPU: transposed operands,
padded leading dimensions, alpha and beta.

Bar: with alpha = 1, beta = 0 the bits of the plain product of op(A), op(B) (the
product is exact before its one rounding, so the storage order cannot change
it); otherwise alpha * AB + beta * C within two ulps of the FP64 evaluation of
that formula; alpha = 0 and beta = 0 read neither the operands nor C.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(torch.device("cuda", 0))


def _ex(h, ta, tb, M, N, K, alpha, A_st, lda, B_st, ldb, beta, C0, ldc):
    import torch
    dA, dB, dC = _dev(A_st), _dev(B_st), _dev(C0)
    rc = h.dgemm_ex(ta, tb, M, N, K, alpha, dA.data_ptr(), lda, dB.data_ptr(), ldb, beta, dC.data_ptr(), ldc,
                    torch.cuda.current_stream().cuda_stream)
    assert rc == 0, h.last_error()
    assert h.sync() == 0, h.last_error()
    return dC.cpu().numpy()


def _store(op, trans, ld_pad):
    """op (rows x cols) stored row-major as op or op^T with ld_pad extra columns."""
    st = op.T if trans else op
    out = np.full((st.shape[0], st.shape[1] + ld_pad), np.nan)
    out[:, :st.shape[1]] = st
    return out, st.shape[1] + ld_pad


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_transposes_bit_identical(gpu_handle, oracle, ta, tb):
    M, N, K = 150, 97, 333
    opA = oracle.gen_phi((M, K), 81, 1.0)
    opB = oracle.gen_phi((K, N), 82, 1.0)
    A_st, lda = _store(opA, ta, 5)
    B_st, ldb = _store(opB, tb, 3)
    C0 = np.full((M, N + 2), np.nan)
    gpu_handle.set_slices(9)
    gpu_handle.set_bins(9)
    C = _ex(gpu_handle, ta, tb, M, N, K, 1.0, A_st, lda, B_st, ldb, 0.0, C0, N + 2)
    ref = oracle.dgemm(opA, opB, 7, 9, 9, 0)
    assert np.array_equal(C[:, :N].view(np.uint64), ref.view(np.uint64))
    assert np.all(np.isnan(C[:, N:]))  # the padding of C is not written


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 1)])
def test_alpha_beta(gpu_handle, oracle, ta, tb):
    M, N, K = 96, 80, 200
    opA = oracle.gen_phi((M, K), 83, 1.0)
    opB = oracle.gen_phi((K, N), 84, 1.0)
    A_st, lda = _store(opA, ta, 0)
    B_st, ldb = _store(opB, tb, 0)
    C0 = oracle.gen_uniform((M, N), 85)
    gpu_handle.set_slices(9)
    gpu_handle.set_bins(9)
    alpha, beta = 2.5, -0.75
    C = _ex(gpu_handle, ta, tb, M, N, K, alpha, A_st, lda, B_st, ldb, beta, C0, N)
    x = oracle.dgemm(opA, opB, 7, 9, 9, 0)
    want = alpha * x + beta * C0
    scale = np.maximum(np.abs(alpha * x), np.abs(beta * C0))
    assert np.all(np.abs(C - want) <= 2 * np.spacing(scale))


def test_alpha_zero_and_beta_zero_read_nothing(gpu_handle, oracle):
    M, N, K = 40, 30, 20
    A = np.full((M, K), np.nan)
    B = np.full((K, N), np.inf)
    C0 = oracle.gen_uniform((M, N), 86)
    C = _ex(gpu_handle, 0, 0, M, N, K, 0.0, A, K, B, N, 3.0, C0, N)
    assert np.array_equal(C, 3.0 * C0)
    opA = oracle.gen_phi((M, K), 87, 1.0)
    opB = oracle.gen_phi((K, N), 88, 1.0)
    C = _ex(gpu_handle, 0, 0, M, N, K, 1.0, opA, K, opB, N, 0.0, np.full((M, N), np.nan), N)
    assert np.all(np.isfinite(C))


def test_bad_leading_dimension(gpu_handle):
    import torch
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = d.data_ptr()
    assert gpu_handle.dgemm_ex(1, 0, 8, 4, 4, 1.0, p, 4, p, 4, 0.0, p, 4) == 7  # lda < M for op(A) = A^T


@pytest.mark.parametrize("M,N,K,rows", [
    (3000, 2048, 256, (0, 1023, 2047, 2048, 2999)),   # 24 row tiles: split after two groups
    (2048, 1104, 256, (0, 1023, 1024, 2047)),         # second launch: 64 tiles, each split along K
])
def test_host_arrays_split_launch_bit_identical(gpu_handle, oracle, ozlib, M, N, K, rows):
    """Host-array calls with more than one group of 8 row tiles run the GEMM as two
    launches and copy the first rows of C back during the second: the result is
    the bits of the device-pointer call (and of the oracle on sampled rows)."""
    import torch
    A = oracle.gen_phi((M, K), 91, 1.0)
    B = oracle.gen_phi((K, N), 92, 1.0)
    gpu_handle.set_slices(9)
    gpu_handle.set_bins(9)
    assert gpu_handle.setup(M, N, K, 1) == 0, gpu_handle.last_error()
    C = np.full((M, N), np.nan)
    for _ in range(2):
        assert gpu_handle.dgemm(M, N, K, A, B, C) == 0, gpu_handle.last_error()
    assert gpu_handle.launch_count() > 0
    h = ozlib.Handle()
    h.set_slices(9)
    h.set_bins(9)
    want = _ex(h, 0, 0, M, N, K, 1.0, A, K, B, N, 0.0, np.full((M, N), np.nan), N)
    h.close()
    assert np.array_equal(C.view(np.uint64), want.view(np.uint64))
    for r0 in rows:
        ref = oracle.dgemm_rows(A, B, 7, 9, 9, 0, r0, r0 + 1)
        assert np.array_equal(C[r0:r0 + 1].view(np.uint64), ref.view(np.uint64)), r0


@pytest.mark.parametrize("ta,tb", [(1, 0), (0, 1), (1, 1)])
def test_transposes_e4m3_slices_bit_identical(gpu_handle, oracle, ta, tb):
    """Transposed operands with 4-bit slices (e4m3 carrier): the transposed split
    jobs keep the oracle's bits."""
    M, N, K = 150, 97, 333
    opA = oracle.gen_phi((M, K), 97, 1.0)
    opB = oracle.gen_phi((K, N), 98, 1.0)
    A_st, lda = _store(opA, ta, 5)
    B_st, ldb = _store(opB, tb, 3)
    gpu_handle.set_bits(4)
    gpu_handle.set_slices(12)
    gpu_handle.set_bins(12)
    C = _ex(gpu_handle, ta, tb, M, N, K, 1.0, A_st, lda, B_st, ldb, 0.0, np.full((M, N), np.nan), N)
    assert gpu_handle.config()["slice_format"] == 1
    ref = oracle.dgemm(opA, opB, 4, 12, 12, 0)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
