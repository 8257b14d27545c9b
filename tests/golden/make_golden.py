"""Writes the golden fixtures in this folder.  Run it where the Oz-AIE sources are
available (it compiles the reference's own host decode through
oracle/build_oracle.py); the outputs are committed and the tests read only them.

    python tests/golden/make_golden.py

Fixtures:
  decode_ref.npz   paired-int64 inputs and the doubles that the reference's compiled
                   convert_paired_i64_to_double_matrix (include/oz_aie.h:92-150)
                   returns for them: pins the restated decode.
  harness.npz      small A, B drawn by the Oz-AIE test-harness formula
                   (test.cpp:219-237, phi in {0.5, 1, 2, 4}) with the exact and the
                   MPFR-106 value of every entry of A B: pins the final results.
  uniform_256x512x128.json     the 256 x 512 x 128 uniform(-1, 1) mt19937_64(0) workload: input
                   digests from the C++ standard library, and digests of every
                   intermediate of the oracle in both profiles, so that the device
                   path can be compared against them without running the oracle.
  uniform_256x512x128_mpfr.npz  the exponents and 64 sampled MPFR-106 values of that workload.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import ozoracle as O  # noqa: E402
import inputs  # noqa: E402


def _gen(tmp, *args):
    exe = os.path.join(tmp, "gen_inputs")
    if not os.path.exists(exe):
        subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(HERE, "gen_inputs.cpp"), "-o", exe])
    out = os.path.join(tmp, "vals.bin")
    subprocess.check_call([exe, *[str(a) for a in args], out])
    return np.fromfile(out, dtype=np.float64)


def decode_cases(rng):
    """Paired-int64 inputs for the decode fixture: the sums of random bins (the
    shape they take in practice) and hand-picked edge patterns."""
    cases = []
    for (M, N, K, b, d) in ((4, 5, 128, 3, 29), (3, 7, 2048, 3, 26), (6, 4, 128, 7, 8), (2, 9, 4096, 7, 8),
                            (5, 5, 1, 4, 18)):
        hi_b = min(2 ** (2 * b) * K, 2 ** 31 - 1)
        bins = rng.integers(-hi_b, hi_b, size=(d, M, N)).astype(np.int64)
        er = rng.integers(900, 1100, size=M).astype(np.int32)
        ec = rng.integers(900, 1100, size=N).astype(np.int32)
        pairs = O.sum_upshift(bins, er, ec, K, b, d)
        cases.append((pairs, K, d, b))
    # edge patterns: zero, +-1 in either word, extreme low words, sign-only high word
    edge = np.array([[0, 0], [1, 0], [-1, 0], [0, 1 << 51], [0, -(1 << 51)], [(1 << 62), 1023 << 51],
                     [-(1 << 62), (1 << 63) | (1023 << 51)], [(1 << 63) - 1, 2046 << 51],
                     [-(1 << 63), 1 << 51], [12345, (1 << 63) | (2000 << 51) | 77]], dtype=object)
    edge = np.array([[int(np.int64(np.uint64(v & 0xFFFFFFFFFFFFFFFF).view(np.int64))) for v in row] for row in edge],
                    dtype=np.int64).reshape(1, -1, 2)
    cases.append((edge, 128, 29, 3))
    cases.append((edge, 512, 8, 7))
    return cases


def make_decode(rng):
    out = {}
    for i, (pairs, K, d, b) in enumerate(decode_cases(rng)):
        ref = O.ref_decode_pairs(pairs, K, d, b)
        if ref is None:
            raise SystemExit("the reference's decode could not be built")
        out["pairs_%d" % i] = pairs
        out["meta_%d" % i] = np.array([K, d, b], np.int64)
        out["out_%d" % i] = ref
    np.savez_compressed(os.path.join(HERE, "decode_ref.npz"), **out)


def make_harness(tmp):
    M, N, K = 24, 32, 40
    out = {"shape": np.array([M, N, K], np.int64)}
    rows, cols = np.meshgrid(np.arange(M, dtype=np.int32), np.arange(N, dtype=np.int32), indexing="ij")
    rows, cols = rows.ravel(), cols.ravel()
    for i, fi in enumerate((0.5, 1.0, 2.0, 4.0)):
        v = _gen(tmp, "harness", i + 1, fi, M * K + K * N)
        A = v[:M * K].reshape(M, K)
        B = v[M * K:].reshape(K, N)
        exact, _ = O.exact_entries(A, B, rows, cols)
        mp = O.mpfr_entries(A, B, rows, cols)
        if mp is None:
            raise SystemExit("libmpfr.so.6 not found")
        tag = "fi%g" % fi
        out["A_" + tag] = A
        out["B_" + tag] = B
        out["exact_" + tag] = exact.reshape(M, N)
        out["mpfr_" + tag] = mp.reshape(M, N)
    np.savez_compressed(os.path.join(HERE, "harness.npz"), **out)


def make_uniform_256x512x128(tmp):
    M, N, K = 256, 512, 128
    v = _gen(tmp, "uniform64", 0, -1.0, 1.0, M * K + K * N)
    A = v[:M * K].reshape(M, K)
    B = v[M * K:].reshape(K, N)
    pa, pb = inputs.uniform_256x512x128_inputs()
    if not (np.array_equal(pa, A) and np.array_equal(pb, B)):
        raise SystemExit("the Python mt19937_64 restatement differs from the C++ standard library")
    H = inputs.sha256
    er, ec = O.max_exp_rows(A), O.max_exp_cols(B)
    doc = {"shape": [M, N, K], "generator": "std::mt19937_64(0), uniform_real_distribution(-1, 1), A then B",
           "A": H(A), "B": H(B), "er": H(er), "ec": H(ec), "profiles": {}}
    # spec profile: b = 7, triangular s = 8 and s = 9, round to nearest
    for s in (8, 9):
        asl = O.split_rows(A, er, 7, s)
        bsl = O.split_cols(B, ec, 7, s)
        bins = O.bins(asl, bsl, s)
        C, q = O.finish(bins, er, ec, 7, 0, want_q=True)
        doc["profiles"]["b7_s%d_tri_rn" % s] = {
            "a_slices": H(asl), "b_slices": H(bsl), "bins": H(bins), "C": H(C), "q": H(q),
            "C_first": [float(x) for x in C.ravel()[:4]]}
    # reference profile: accurate mode for log2 K = 7 -> (b, d) = (3, 29); fast -> (7, 8)
    for name, (b, d) in (("ref_accurate_b3_d29", (3, 29)), ("ref_fast_b7_d8", (7, 8))):
        asl = O.split_rows(A, er, b, d)
        bsl = O.split_cols(B, ec, b, d)
        bins = O.bins(asl, bsl, d)
        pairs = O.sum_upshift(bins, er, ec, K, b, d)
        C = O.ref_decode_pairs(pairs, K, d, b)
        if C is None:
            raise SystemExit("the reference's decode could not be built")
        if not np.array_equal(C.view(np.uint64), O.decode_pairs(pairs, K, d, b).view(np.uint64)):
            raise SystemExit("restated decode differs from the reference's")
        doc["profiles"][name] = {"a_slices": H(asl), "b_slices": H(bsl), "bins": H(bins), "pairs": H(pairs),
                                 "C": H(C), "C_first": [float(x) for x in C.ravel()[:4]]}
    r, c = O.sample_indices(M, N, 64, 11)
    mp = O.mpfr_entries(A, B, r, c)
    if mp is None:
        raise SystemExit("libmpfr.so.6 not found")
    np.savez_compressed(os.path.join(HERE, "uniform_256x512x128_mpfr.npz"), er=er, ec=ec, rows=r, cols=c, mpfr=mp)
    with open(os.path.join(HERE, "uniform_256x512x128.json"), "w") as f:
        json.dump(doc, f, indent=1)
        f.write("\n")


def main():
    rng = np.random.default_rng(20240611)
    with tempfile.TemporaryDirectory() as tmp:
        make_decode(rng)
        make_harness(tmp)
        make_uniform_256x512x128(tmp)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
