"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle.

Bar: bit-exact for the integer stages (exponents, int8 slices, exact bin sums);
bit-exact FP64 results in both rounding modes (the oracle applies the same
finishing rule to the same exact integers); the reference's truncating decode
matched bit for bit in its own configuration.
"""
import numpy as np
import pytest

from ozaie_gb300.api import q_words_to_int

pytestmark = pytest.mark.gpu

FAST = 1


def _run(h, A, B, mode=FAST):
    M, K = A.shape
    N = B.shape[1]
    assert h.setup(M, N, K, mode) == 0, h.last_error()
    C = np.empty((M, N))
    assert h.dgemm(M, N, K, np.ascontiguousarray(A), np.ascontiguousarray(B), C) == 0, h.last_error()
    return C


def _oracle_q(O, A, B, b, s, J):
    er, ec = O.max_exp_rows(A), O.max_exp_cols(B)
    bins = O.bins(O.split_rows(A, er, b, s), O.split_cols(B, ec, b, s), J)
    return er, ec, bins


def _q_from_bins(bins, b, J):
    out = np.zeros(bins.shape[1:], dtype=object)
    for j in range(J):
        out = out + bins[j].astype(object) * (1 << (b * (J - 1 - j)))
    return out


@pytest.mark.parametrize("shape,b,s,J", [
    ((256, 512, 128), 7, 8, 8),
    ((256, 512, 128), 3, 29, 29),
    ((130, 70, 200), 7, 9, 9),
    ((64, 48, 96), 7, 8, 15),
    ((1, 1, 1), 7, 8, 8),
    ((33, 17, 45), 5, 11, 11),
])
def test_slices_and_exponents_bit_exact(gpu_handle, oracle, shape, b, s, J):
    M, N, K = shape
    A = oracle.gen_phi((M, K), 1, 2.0)
    B = oracle.gen_phi((K, N), 2, 2.0)
    gpu_handle.set_bits(b)
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(J)
    d = gpu_handle.dump(A, B, want_q=False)
    er, ec = oracle.max_exp_rows(A), oracle.max_exp_cols(B)
    assert np.array_equal(d["er"], er)
    assert np.array_equal(d["ec"], ec)
    assert np.array_equal(d["a_slices"], oracle.split_rows(A, er, b, s))
    assert np.array_equal(d["b_slices"], oracle.split_cols(B, ec, b, s))


@pytest.mark.parametrize("shape,b,s,J", [
    ((256, 512, 128), 7, 8, 8),
    ((128, 64, 1000), 7, 8, 8),      # K spans several exact-drain periods
    ((100, 96, 777), 7, 9, 9),
    ((64, 64, 300), 7, 6, 11),       # between triangular and full
    ((96, 40, 250), 7, 8, 15),       # full pair set, 4-word accumulator
    ((256, 128, 128), 3, 29, 29),    # the reference's accurate table at K=128
])
def test_exact_accumulator_matches_bins(gpu_handle, oracle, shape, b, s, J):
    M, N, K = shape
    A = oracle.gen_phi((M, K), 3, 1.0)
    B = oracle.gen_phi((K, N), 4, 1.0)
    gpu_handle.set_bits(b)
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(J)
    d = gpu_handle.dump(A, B, want_slices=False)
    _, _, bins = _oracle_q(oracle, A, B, b, s, J)
    q_gpu = q_words_to_int(d["q"])
    q_ref = _q_from_bins(bins, b, J)
    assert (q_gpu == q_ref).all()


@pytest.mark.parametrize("j", [0, 3, 7])
def test_single_bin_bit_exact(gpu_handle, oracle, j):
    """One bin at a time: the int32 partial products of the reference (bins) exactly."""
    M, N, K, b, s = 128, 64, 256, 7, 8
    A = oracle.gen_uniform((M, K), 5)
    B = oracle.gen_uniform((K, N), 6)
    gpu_handle.set_bits(b)
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(s)
    d = gpu_handle.dump(A, B, bin_lo=j, bin_hi=j, want_slices=False)
    _, _, bins = _oracle_q(oracle, A, B, b, s, s)
    q = q_words_to_int(d["q"])
    shift = 1 << (b * (s - 1 - j))
    assert (q % shift == 0).all()
    got = (q // shift).astype(np.int64)
    assert np.array_equal(got, bins[j])
    # the reference keeps bins in int32: identical whenever no wrap occurs
    assert np.array_equal(got.astype(np.int32).astype(np.int64), bins[j])


def test_reference_profile_bit_exact(gpu_handle, oracle):
    """Reference tables + truncating decode: identical bits to the reference's
    device sum + host decode (oracle restatement, whose decode is pinned to the
    reference's own compiled function)."""
    M, N, K = 256, 512, 128
    A = oracle.gen_uniform((M, K), 0)
    B = oracle.gen_uniform((K, N), 1)
    gpu_handle.set_profile(1)
    for mode, (b, d) in ((0, (3, 29)), (1, (7, 8))):
        C = _run(gpu_handle, A, B, mode)
        cfg = gpu_handle.config()
        assert (cfg["bits"], cfg["slices"], cfg["bins"]) == (b, d, d)
        er, ec, bins = _oracle_q(oracle, A, B, b, d, d)
        pairs = oracle.sum_upshift(bins, er, ec, K, b, d)
        ref = oracle.decode_pairs(pairs, K, d, b)
        assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("shape,s,J,phi", [
    ((256, 512, 128), 8, 8, 1.0),
    ((200, 136, 300), 9, 9, 0.5),
    ((77, 91, 513), 8, 15, 4.0),
    ((5, 3, 2), 8, 8, 1.0),
])
def test_round_to_nearest_bit_exact(gpu_handle, oracle, shape, s, J, phi):
    M, N, K = shape
    A = oracle.gen_phi((M, K), 7, phi)
    B = oracle.gen_phi((K, N), 8, phi)
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(J)
    C = _run(gpu_handle, A, B)
    ref = oracle.dgemm(A, B, 7, s, J, 0)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))


def test_nearest_vs_reference_decode_within_one_ulp(gpu_handle, oracle):
    M, N, K = 128, 128, 256
    A = oracle.gen_phi((M, K), 9, 1.0)
    B = oracle.gen_phi((K, N), 10, 1.0)
    gpu_handle.set_slices(8)
    gpu_handle.set_bins(8)
    gpu_handle.set_rounding(0)
    rn = _run(gpu_handle, A, B)
    gpu_handle.set_rounding(1)
    rz = _run(gpu_handle, A, B)
    assert np.max(np.abs(rn.view(np.int64) - rz.view(np.int64))) <= 1


def test_adversarial_exactness_at_drain_boundary(gpu_handle, oracle):
    """All slices +-127 (every product 16129) across a full exact-drain period,
    mixed with tiny entries whose low-order contributions must survive."""
    M, N, K = 128, 64, 1024
    big = np.float64(np.frombuffer(np.uint64(0x3FFFFFFFFFFFFFFF).tobytes(), np.float64)[0])  # 1.999...
    A = np.full((M, K), big)
    B = np.full((K, N), big)
    A[::3, ::5] = -big
    B[1::4, ::7] = 2.0 ** -30
    A[5, 7] = 2.0 ** -40
    gpu_handle.set_slices(8)
    gpu_handle.set_bins(8)
    d = gpu_handle.dump(A, B, want_slices=False)
    _, _, bins = _oracle_q(oracle, A, B, 7, 8, 8)
    assert (q_words_to_int(d["q"]) == _q_from_bins(bins, 7, 8)).all()
    C = _run(gpu_handle, A, B)
    assert np.array_equal(C.view(np.uint64), oracle.dgemm(A, B, 7, 8, 8, 0).view(np.uint64))


def test_zero_and_special_rows(gpu_handle, oracle):
    M, N, K = 64, 64, 64
    A = oracle.gen_uniform((M, K), 12)
    B = oracle.gen_uniform((K, N), 13)
    A[3] = 0.0
    A[4, :] = 5e-324  # subnormals: the reference's bias quirk
    B[:, 9] = -0.0
    gpu_handle.set_slices(8)
    gpu_handle.set_bins(8)
    C = _run(gpu_handle, A, B)
    ref = oracle.dgemm(A, B, 7, 8, 8, 0)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
    assert np.all(C[3] == 0.0)


def test_accuracy_vs_exact_s9(gpu_handle, oracle):
    M, N, K = 384, 384, 1024
    A = oracle.gen_phi((M, K), 21, 1.0)
    B = oracle.gen_phi((K, N), 22, 1.0)
    gpu_handle.set_slices(9)
    gpu_handle.set_bins(9)
    C = _run(gpu_handle, A, B)
    r, c = oracle.sample_indices(M, N, 1000, 5)
    e = oracle.error_report(C, A, B, r, c)
    assert e["normwise_rel"] <= 1e-15, e


def test_device_timeout_path_is_recoverable(gpu_handle, oracle):
    """A wait on an mbarrier nothing arrives on gives up after its limit and the
    context stays usable."""
    assert gpu_handle.selftest_timeout(20.0) == 9  # OZGB_ERR_TIMEOUT
    A = oracle.gen_uniform((32, 32), 1)
    B = oracle.gen_uniform((32, 32), 2)
    gpu_handle.set_slices(8)
    gpu_handle.set_bins(8)
    C = _run(gpu_handle, A, B)
    assert np.array_equal(C.view(np.uint64), oracle.dgemm(A, B, 7, 8, 8, 0).view(np.uint64))


@pytest.mark.parametrize("mode,shape", [(0, (256, 512, 128)), (1, (256, 512, 128)), (0, (130, 70, 1024)),
                                        (1, (77, 91, 2048))])
def test_reference_device_output_pairs(gpu_handle, oracle, mode, shape):
    """The reference profile's paired int64 output equals the oracle's restatement
    of the reference's device sum bit for bit, and decodes (with the reference's
    host decode, pinned) to the profile's final results."""
    M, N, K = shape
    A = oracle.gen_phi((M, K), 71, 1.0)
    B = oracle.gen_phi((K, N), 72, 1.0)
    gpu_handle.set_profile(1)
    C = _run(gpu_handle, A, B, mode)
    cfg = gpu_handle.config()
    b, d = cfg["bits"], cfg["slices"]
    pairs = gpu_handle.dump_pairs(A, B)
    er, ec, bins = _oracle_q(oracle, A, B, b, d, d)
    want = oracle.sum_upshift(bins, er, ec, K, b, d)
    assert np.array_equal(pairs, want)
    assert np.array_equal(oracle.decode_pairs(pairs, K, d, b).view(np.uint64), C.view(np.uint64))


@pytest.mark.parametrize("b,s,J", [(4, 10, 10), (3, 18, 18), (4, 8, 15), (2, 12, 12)])
def test_e4m3_carrier_bit_exact(gpu_handle, oracle, b, s, J):
    """Slices of b <= 4 bits run on e4m3 (kind::f8f6f4, 64 K values per chunk): the
    result keeps the oracle's bits, through several drains and the K-split."""
    import torch
    M, N, K = 300, 200, 3000
    A = oracle.gen_phi((M, K), 95, 1.0)
    B = oracle.gen_phi((K, N), 96, 1.0)
    dev = torch.device("cuda", 0)
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    dC = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
    gpu_handle.set_bits(b)
    gpu_handle.set_slices(s)
    gpu_handle.set_bins(J)
    assert gpu_handle.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N,
                                   torch.cuda.current_stream().cuda_stream) == 0, gpu_handle.last_error()
    assert gpu_handle.sync() == 0, gpu_handle.last_error()
    cfg = gpu_handle.config()
    assert cfg["slice_format"] == 1
    ref = oracle.dgemm(A, B, b, s, J, 0)
    assert np.array_equal(dC.cpu().numpy().view(np.uint64), ref.view(np.uint64))
