"""CPU tests of the oracle: against the reference's own compiled decode, the golden
fixtures, and independent big-integer restatements of the reference's split,
bin-product and device-sum arithmetic.

These pin the checker that the GPU parity tests use; no GPU is needed.
"""
import json
import os
from fractions import Fraction

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ------------------------------------------------- independent restatements
def split_restated(x, E, b, d):
    """Slices of double x against the exponent field E, following the word-level
    steps of ozaki_base.cc:490-629 with Python integers: four 32-bit words selected
    by bias >= 32/64/96 (the fourth not cleared past 128, :543-544), the 128-bit
    window shifted right by bias mod 32 (:551), slices read MSB first (:581-629)."""
    bits = int(np.float64(x).view(np.uint64))
    sg, e, f = bits >> 63, (bits >> 52) & 0x7FF, bits & ((1 << 52) - 1)
    hi32, lo32 = f >> 32, f & 0xFFFFFFFF
    if e != 0:
        hi32 += 1 << 20
    bias = (E - e) & 0xFFFFFFFF
    hi = ((hi32 << 11) | (lo32 >> 21)) & 0xFFFFFFFF
    lo = (lo32 << 11) & 0xFFFFFFFF
    avoid = 1 + (3 if b == 3 else 0)
    nv0 = 64 - avoid - ((64 - avoid) % b)
    two = d * b > nv0
    w0 = 0 if bias >= 32 else hi
    w1 = 0 if bias >= 64 else (hi if bias >= 32 else lo)
    w2 = w3 = 0
    if two:
        w2 = 0 if bias >= 96 else (hi if bias >= 64 else (lo if bias >= 32 else 0))
        w3 = hi if bias >= 96 else (lo if bias >= 64 else 0)
    V = ((w0 << 96) | (w1 << 64) | (w2 << 32) | w3) >> (bias & 31)
    if not two:
        V = (V >> 64) << 64
    out = []
    for i in range(d):
        v = (V >> (128 - b * (i + 1))) & ((1 << b) - 1)
        out.append(-v if sg else v)
    return out


def first_group_restated(K, b, d):
    """ozaki_base.cc:151-158 with log2 K = countr_zero(K) (include/oz_aie.h:100)."""
    log2k = (K & -K).bit_length() - 1
    numer = b * (d + 1) - 51 + log2k
    g_min = 1 if numer < 0 else numer // b + 1
    return min(d, max(g_min, 31 // b + 1))


def sum_upshift_restated(bins, er, ec, K, b, d):
    """ozaki_base.cc:279-328: lo and hi int64 words with (Er + Ec) embedded in bits
    51..62 of hi, the sign bit kept."""
    g0 = first_group_restated(K, b, d)
    J, M, N = bins.shape
    out = np.zeros((M, N, 2), np.int64)
    for r in range(M):
        for c in range(N):
            lo = sum(int(bins[d - 1 - t, r, c]) << (b * t) for t in range(g0))
            hi = sum(int(bins[d - 1 - g0 - t, r, c]) << (b * t) for t in range(d - g0))
            lo &= (1 << 64) - 1
            hi &= (1 << 64) - 1
            hi = (hi & ((1 << 51) - 1)) | (hi & (1 << 63)) | ((int(er[r]) + int(ec[c])) << 51)
            out[r, c, 0] = np.uint64(lo).view(np.int64)
            out[r, c, 1] = np.uint64(hi).view(np.int64)
    return out


def nearest_double(fr):
    """Round a Fraction to the nearest double, ties to even (Python's own
    correctly rounded int / int division)."""
    return float(fr.numerator / fr.denominator) if fr else 0.0


# ------------------------------------------------------------- decode pins
def _decode_cases():
    z = np.load(os.path.join(GOLDEN, "decode_ref.npz"))
    n = len([k for k in z.files if k.startswith("pairs_")])
    return [(z["pairs_%d" % i], *[int(v) for v in z["meta_%d" % i]], z["out_%d" % i]) for i in range(n)]


def test_decode_matches_reference_fixture(oracle):
    for pairs, K, d, b, ref in _decode_cases():
        got = oracle.decode_pairs(pairs, K, d, b)
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (K, d, b)


def test_library_decode_matches_reference_fixture(ozlib):
    from ozaie_gb300.api import convert_paired_i64_to_double_matrix
    for pairs, K, d, b, ref in _decode_cases():
        M, N, _ = pairs.shape
        out = np.zeros(M * N)
        convert_paired_i64_to_double_matrix(pairs.ravel(), out, M, N, K, d, b)
        assert np.array_equal(out.view(np.uint64), ref.ravel().view(np.uint64)), (K, d, b)


def test_decode_matches_live_reference(oracle):
    """Where the reference's sources are present, its compiled decode against the
    restatement on fresh random sums."""
    if oracle.ref_decode_lib() is None:
        pytest.skip("reference decode not built (sources absent)")
    rng = np.random.default_rng(5)
    for (K, b, d) in ((128, 3, 29), (1024, 3, 27), (4096, 7, 8), (64, 7, 9)):
        bins = rng.integers(-(1 << 2 * b) * K, (1 << 2 * b) * K, size=(d, 9, 11)).astype(np.int64)
        er = rng.integers(1, 2046, 9).astype(np.int32) // 2
        ec = rng.integers(1, 2046, 11).astype(np.int32) // 2
        pairs = oracle.sum_upshift(bins, er, ec, K, b, d)
        a = oracle.decode_pairs(pairs, K, d, b)
        r = oracle.ref_decode_pairs(pairs, K, d, b)
        assert np.array_equal(a.view(np.uint64), r.view(np.uint64))


# ------------------------------------------------------- split restatement
SPLIT_CASES = [(7, 8), (7, 9), (3, 29), (3, 27), (5, 11), (4, 18), (7, 16), (6, 12)]


@pytest.mark.parametrize("b,d", SPLIT_CASES)
def test_split_matches_word_level_restatement(oracle, b, d):
    rng = np.random.default_rng(b * 100 + d)
    xs = list(oracle.gen_phi(300, b + d, 2.0))
    xs += [0.0, -0.0, 1.0, -1.0, 5e-324, -2.2250738585072014e-308, 1.7976931348623157e308, 2.0 ** -1022,
           np.nextafter(1.0, 2.0), -np.nextafter(2.0, 0.0)]
    for x in xs:
        e = (int(np.float64(x).view(np.uint64)) >> 52) & 0x7FF
        # exponents at and above the element's own, including distances past 64 and 128
        for E in sorted({e, e + 1, e + 7, e + 31, e + 32, e + 33, e + 63, e + 64, e + 65, e + 100, e + 127,
                         e + 128, e + 140, min(2046, e + int(rng.integers(0, 60)))}):
            if E > 2047:
                continue
            got = [int(v) for v in oracle.split_values(np.array([x]), E, b, d)[0]]
            assert got == split_restated(x, E, b, d), (x, E, b, d)


def test_split_planes_match_elementwise(oracle):
    A = oracle.gen_phi((13, 21), 3, 1.5)
    er = oracle.max_exp_rows(A)
    P = oracle.split_rows(A, er, 7, 9)
    for r in range(13):
        for k in range(21):
            assert list(P[:, r, k]) == split_restated(A[r, k], int(er[r]), 7, 9)
    B = oracle.gen_phi((21, 10), 4, 1.5)
    ec = oracle.max_exp_cols(B)
    Q = oracle.split_cols(B, ec, 3, 29)
    for k in range(21):
        for c in range(10):
            assert list(Q[:, k, c]) == split_restated(B[k, c], int(ec[c]), 3, 29)


def test_split_is_a_truncation(oracle):
    """x - sum_i slice_i 2^(E - 1022 - b(i+1)) has the sign of x (or is 0) and is
    below one unit of the last slice: the split is error-free up to truncation."""
    xs = oracle.gen_phi(500, 9, 1.0)
    E = (xs.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    Emax = int(E.max())
    b, d = 7, 9
    P = oracle.split_values(xs, Emax, b, d)
    for x, sl in zip(xs, P):
        approx = sum(Fraction(int(v)) * Fraction(2) ** (Emax - 1022 - b * (i + 1)) for i, v in enumerate(sl))
        rem = Fraction(float(x)) - approx
        assert rem == 0 or (rem > 0) == (x > 0)
        assert abs(rem) < Fraction(2) ** (Emax - 1022 - b * d)


def test_exponents_are_field_maxima(oracle):
    A = oracle.gen_phi((17, 33), 1, 3.0)
    A[3] = 0.0
    A[5, :4] = 5e-324
    f = ((A.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    assert np.array_equal(oracle.max_exp_rows(A), f.max(axis=1))
    assert np.array_equal(oracle.max_exp_cols(A), f.max(axis=0))


# ----------------------------------------------------- products and sums
@pytest.mark.parametrize("d,J", [(8, 8), (9, 9), (8, 15), (5, 3)])
def test_bins_match_integer_matmul(oracle, d, J):
    rng = np.random.default_rng(d * J)
    Ap = rng.integers(-127, 128, size=(d, 11, 37)).astype(np.int8)
    Bp = rng.integers(-127, 128, size=(d, 37, 13)).astype(np.int8)
    got = oracle.bins(Ap, Bp, J)
    for j in range(J):
        want = np.zeros((11, 13), np.int64)
        for p in range(d):
            q = j - p
            if 0 <= q < d:
                want += Ap[p].astype(np.int64) @ Bp[q].astype(np.int64)
        assert np.array_equal(got[j], want), j


def test_first_group_formula(oracle):
    for b in range(2, 9):
        for d in range(1, 40):
            for K in (1, 2, 64, 128, 1000, 2048, 4096, 65536):
                assert oracle.first_group(K, b, d) == first_group_restated(K, b, d), (K, b, d)


@pytest.mark.parametrize("K,b,d", [(128, 3, 29), (2048, 3, 26), (4096, 7, 8), (128, 7, 8)])
def test_sum_upshift_matches_restatement(oracle, K, b, d):
    rng = np.random.default_rng(K + b + d)
    lim = min((1 << 2 * b) * K, (1 << 31) - 1)
    bins = rng.integers(-lim, lim, size=(d, 4, 6)).astype(np.int64)
    er = rng.integers(800, 1200, 4).astype(np.int32)
    ec = rng.integers(800, 1200, 6).astype(np.int32)
    assert np.array_equal(oracle.sum_upshift(bins, er, ec, K, b, d), sum_upshift_restated(bins, er, ec, K, b, d))


@pytest.mark.parametrize("J,b", [(8, 7), (15, 7), (29, 3)])
def test_finish_round_to_nearest(oracle, J, b):
    """RN finish = the exact value q 2^(Er+Ec-2044-b(J+1)), q = sum_j bin_j 2^(b(J-1-j)),
    correctly rounded."""
    rng = np.random.default_rng(J)
    bins = rng.integers(-(1 << 20), 1 << 20, size=(J, 3, 5)).astype(np.int64)
    er = rng.integers(1000, 1040, 3).astype(np.int32)
    ec = rng.integers(1000, 1040, 5).astype(np.int32)
    C = oracle.finish(bins, er, ec, b, rounding=0)
    for r in range(3):
        for c in range(5):
            q = sum(int(bins[j, r, c]) << (b * (J - 1 - j)) for j in range(J))
            v = Fraction(q) * Fraction(2) ** (int(er[r]) + int(ec[c]) - 2044 - b * (J + 1))
            assert C[r, c] == nearest_double(v)


def test_exact_entries_are_correctly_rounded(oracle):
    A = oracle.gen_phi((6, 50), 1, 3.0)
    B = oracle.gen_phi((50, 7), 2, 3.0)
    rows = np.repeat(np.arange(6, dtype=np.int32), 7)
    cols = np.tile(np.arange(7, dtype=np.int32), 6)
    got, _ = oracle.exact_entries(A, B, rows, cols)
    for i, (r, c) in enumerate(zip(rows, cols)):
        s = sum(Fraction(float(A[r, k])) * Fraction(float(B[k, c])) for k in range(50))
        assert got[i] == nearest_double(s)


# ------------------------------------------------------------ golden fixtures
def test_uniform_256x512x128_generator_matches_cpp_fixture():
    from golden import inputs
    doc = json.load(open(os.path.join(GOLDEN, "uniform_256x512x128.json")))
    A, B = inputs.uniform_256x512x128_inputs()
    assert inputs.sha256(A) == doc["A"] and inputs.sha256(B) == doc["B"]


def test_uniform_256x512x128_oracle_intermediates(oracle):
    """Every oracle intermediate of the 256 x 512 x 128 workload against the
    committed digests (made where the reference's decode was compiled)."""
    from golden import inputs
    H = inputs.sha256
    doc = json.load(open(os.path.join(GOLDEN, "uniform_256x512x128.json")))
    A, B = inputs.uniform_256x512x128_inputs()
    M, N, K = doc["shape"]
    er, ec = oracle.max_exp_rows(A), oracle.max_exp_cols(B)
    assert H(er) == doc["er"] and H(ec) == doc["ec"]
    for s in (8, 9):
        want = doc["profiles"]["b7_s%d_tri_rn" % s]
        asl, bsl = oracle.split_rows(A, er, 7, s), oracle.split_cols(B, ec, 7, s)
        bins = oracle.bins(asl, bsl, s)
        C, q = oracle.finish(bins, er, ec, 7, 0, want_q=True)
        assert [H(asl), H(bsl), H(bins), H(C), H(q)] == [want[k] for k in ("a_slices", "b_slices", "bins", "C", "q")]
    for name, (b, d) in (("ref_accurate_b3_d29", (3, 29)), ("ref_fast_b7_d8", (7, 8))):
        want = doc["profiles"][name]
        asl, bsl = oracle.split_rows(A, er, b, d), oracle.split_cols(B, ec, b, d)
        bins = oracle.bins(asl, bsl, d)
        pairs = oracle.sum_upshift(bins, er, ec, K, b, d)
        C = oracle.decode_pairs(pairs, K, d, b)
        assert [H(asl), H(bsl), H(bins), H(pairs), H(C)] == \
            [want[k] for k in ("a_slices", "b_slices", "bins", "pairs", "C")]


def test_uniform_256x512x128_results_against_mpfr(oracle):
    """The reference's correctness gate (common.h:338-341: relative 0.05 or absolute
    0.5 against MPFR-106) and the tighter bound of this library."""
    from golden import inputs
    z = np.load(os.path.join(GOLDEN, "uniform_256x512x128_mpfr.npz"))
    A, B = inputs.uniform_256x512x128_inputs()
    r, c, mp = z["rows"], z["cols"], z["mpfr"]
    ref_acc = oracle.dgemm(A, B, 3, 29, 29, 1)[r, c]
    assert np.all((np.abs(ref_acc - mp) <= 0.5) | (np.abs(ref_acc - mp) <= 0.05 * np.abs(mp)))
    assert np.max(np.abs(ref_acc - mp) / np.abs(mp)) < 1e-14
    rn9 = oracle.dgemm(A, B, 7, 9, 9, 0)[r, c]
    assert np.linalg.norm(rn9 - mp) / np.linalg.norm(mp) <= 1e-15


@pytest.mark.parametrize("fi", [0.5, 1.0, 2.0, 4.0])
def test_harness_fixture_exact_and_mpfr(oracle, fi):
    z = np.load(os.path.join(GOLDEN, "harness.npz"))
    tag = "fi%g" % fi
    A, B, exact, mp = z["A_" + tag], z["B_" + tag], z["exact_" + tag], z["mpfr_" + tag]
    M, N, K = [int(v) for v in z["shape"]]
    rows = np.repeat(np.arange(M, dtype=np.int32), N)
    cols = np.tile(np.arange(N, dtype=np.int32), M)
    got, _ = oracle.exact_entries(A, B, rows, cols)
    assert np.array_equal(got.reshape(M, N), exact)
    # MPFR-106 accumulates with rounding: it may differ from the exact value by a few ulps
    assert np.max(np.abs(mp - exact) / np.maximum(np.abs(exact), 1e-300)) < 1e-12
    # accurate enough slices give the exact result to within the stated bound
    s = {0.5: 9, 1.0: 9, 2.0: 11, 4.0: 15}[fi]
    C = oracle.dgemm(A, B, 7, s, s, 0)
    assert np.linalg.norm(C - exact) / np.linalg.norm(exact) <= 1e-15
