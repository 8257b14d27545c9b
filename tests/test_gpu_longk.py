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


def test_split_wave_alpha_beta_and_reference_decode(ozlib, oracle):
    """The K-split's completing part runs the same epilogue as a whole tile: with
    C = alpha AB + beta C (beta read once) and with the reference's truncating
    decode (reference profile, e4m3 slices of 3 bits)."""
    import torch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream().cuda_stream
    # 12 tiles of 128 x 48 with 64 chunks: each tile split along K
    M, N, K = 256, 288, 2048
    A = oracle.gen_phi((M, K), 51, 1.0)
    B = oracle.gen_phi((K, N), 52, 1.0)
    C0 = oracle.gen_uniform((M, N), 53)
    dA, dB, dC = (torch.from_numpy(x).to(dev) for x in (A, B, C0))
    h = ozlib.Handle()
    h.set_slices(9)
    h.set_bins(9)
    alpha, beta = -1.5, 0.25
    assert h.dgemm_ex(0, 0, M, N, K, alpha, dA.data_ptr(), K, dB.data_ptr(), N, beta, dC.data_ptr(), N, stream) == 0
    assert h.sync() == 0, h.last_error()
    h.close()
    x = oracle.dgemm(A, B, 7, 9, 9, 0)
    want = alpha * x + beta * C0
    scale = np.maximum(np.abs(alpha * x), np.abs(beta * C0))
    assert np.all(np.abs(dC.cpu().numpy() - want) <= 2 * np.spacing(scale))
    # reference profile: K = 4096 picks (b, d) = (3, 25) from the reference's table
    M, N, K = 128, 384, 4096
    A = oracle.gen_phi((M, K), 54, 1.0)
    B = oracle.gen_phi((K, N), 55, 1.0)
    h = ozlib.Handle()
    h.set_profile(1)
    assert h.setup(M, N, K, 0) == 0, h.last_error()
    C = np.empty((M, N))
    assert h.dgemm(M, N, K, A, B, C) == 0, h.last_error()
    cfg = h.config()
    h.close()
    assert cfg["slice_format"] == 1 and cfg["bits"] == 3
    ref = oracle.dgemm(A, B, cfg["bits"], cfg["slices"], cfg["bins"], 1)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
