"""Long inner dimension and ill-conditioned rows on the GPU.

K = 65536 forces many drains of the fp32 accumulators into the exact integer
accumulator (the K-blocking of the long-K workload); rows of A scaled by
2^(-40 i / M) exercise per-row exponents over a wide range.  Bar: bit-identical
to the oracle on the rows it can afford, and within the bound of the exact
products on sampled entries.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_dgemm(ozlib, A, B, s=None, J=None, bound=None):
    import torch
    dev = torch.device("cuda", 0)
    M, K = A.shape
    N = B.shape[1]
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    dC = torch.empty((M, N), dtype=torch.float64, device=dev)
    h = ozlib.Handle()
    if s:
        h.set_slices(s)
        h.set_bins(J or s)
    if bound:
        h.set_error_bound(bound)
    rc = h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N,
                        torch.cuda.current_stream().cuda_stream)
    assert rc == 0, h.last_error()
    assert h.sync() == 0, h.last_error()
    cfg = h.config()
    h.close()
    return dC.cpu().numpy(), cfg


@pytest.mark.parametrize("s,J", [(9, 9), (8, 15)])
def test_long_k_rows_bit_exact(ozlib, oracle, s, J):
    M, N, K = 256, 192, 65536
    A = oracle.gen_phi((M, K), 41, 1.0)
    B = oracle.gen_phi((K, N), 42, 1.0)
    C, cfg = _device_dgemm(ozlib, A, B, s, J)
    assert cfg["k_chunk"] * cfg["drain_chunks"] < K  # many drains per tile
    for r0 in (0, 131, 255):
        ref = oracle.dgemm_rows(A, B, 7, s, J, 0, r0, r0 + 1)
        assert np.array_equal(C[r0:r0 + 1].view(np.uint64), ref.view(np.uint64)), r0


def test_long_k_adaptive_accuracy(ozlib, oracle):
    M, N, K = 256, 256, 65536
    A = oracle.gen_phi((M, K), 43, 1.0)
    B = oracle.gen_phi((K, N), 44, 1.0)
    C, cfg = _device_dgemm(ozlib, A, B, bound=1e-15)
    r, c = oracle.sample_indices(M, N, 256, 5)
    exact, _ = oracle.exact_entries(A, B, r, c)
    assert np.linalg.norm(C[r, c] - exact) / np.linalg.norm(exact) <= 1e-15


def test_ill_conditioned_rows(ozlib, oracle):
    """Row i of A scaled by 2^(-40 i / M), the ill-conditioned variant of the
    long-K workload: per-row exponents keep every row at full relative accuracy."""
    M, N, K = 512, 256, 4096
    A = oracle.gen_phi((M, K), 45, 1.0) * np.exp2(-40.0 * np.arange(M) / M)[:, None]
    B = oracle.gen_phi((K, N), 46, 1.0)
    C, _ = _device_dgemm(ozlib, A, B, 9, 9)
    for r0 in (0, 300, 511):
        ref = oracle.dgemm_rows(A, B, 7, 9, 9, 0, r0, r0 + 1)
        assert np.array_equal(C[r0:r0 + 1].view(np.uint64), ref.view(np.uint64)), r0
    rows = np.repeat(np.array([0, 255, 511], np.int32), 64)
    cols = np.tile(np.arange(64, dtype=np.int32), 3)
    exact, _ = oracle.exact_entries(A, B, rows, cols)
    for i in range(3):
        sl = slice(64 * i, 64 * (i + 1))
        got = C[rows[sl], cols[sl]]
        assert np.linalg.norm(got - exact[sl]) / np.linalg.norm(exact[sl]) <= 1e-15


def test_partial_wave_split_bit_exact(ozlib, oracle):
    """156 tiles of 128 x 48 on a 152-SM GPU: the last wave's 4 tiles are split
    into K parts whose exact group sums are added in global memory; every row,
    including the rows of the split tiles (rows 1152-1663, columns 528-575), keeps
    the oracle's bits."""
    import torch
    M, N, K = 1664, 576, 2048
    A = oracle.gen_phi((M, K), 47, 1.0)
    B = oracle.gen_phi((K, N), 48, 1.0)
    dev = torch.device("cuda", 0)
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    h = ozlib.Handle()
    h.set_slices(9)
    h.set_bins(9)
    refs = {r0: oracle.dgemm_rows(A, B, 7, 9, 9, 0, r0, r0 + 1) for r0 in (0, 700, 1152, 1300, 1663)}
    # three calls on one handle: the later ones use the scratch the earlier ones left zero
    for _ in range(3):
        dC = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
        assert h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N,
                              torch.cuda.current_stream().cuda_stream) == 0, h.last_error()
        assert h.sync() == 0, h.last_error()
        assert h.config()["tile_n"] == 48
        C = dC.cpu().numpy()
        for r0, ref in refs.items():
            assert np.array_equal(C[r0:r0 + 1].view(np.uint64), ref.view(np.uint64)), r0
    h.close()
