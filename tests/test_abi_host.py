"""CPU tests of the C ABI: the library loads and exports every declared symbol, the
headers compile, the host-only entry points (planning, precision knob, decode)
behave, and calls without a GPU fail with status codes instead of crashing.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import HAVE_GPU, ROOT

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in os.listdir(INCLUDE):
        if h.endswith(".h") and h != "oz_aie.h":
            text = open(os.path.join(INCLUDE, h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(ozgb_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(ozlib):
    from ozaie_gb300 import _lib
    lib = ctypes.CDLL(_lib.lib_path())
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(names) <= bound, set(names) - bound


def test_c_header_compiles_as_c99_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "oz_gb300.h"\nint main(void) { ozgb_handle h = 0; (void)h; return 0; }\n')
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", INCLUDE, str(src)])
    cpp = tmp_path / "t.cpp"
    cpp.write_text('#include "oz_aie.h"\n#include "oz_aie.h"\nint main() { return oz_aie::Mode::fast; }\n')
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", INCLUDE, str(cpp)])


def test_dropin_example_builds_and_runs(ozlib, tmp_path):
    """example/oztest.cpp, the reference's usage, against the drop-in header: it
    links, and without a GPU it stops at setup with status 2."""
    from ozaie_gb300 import _lib
    exe = tmp_path / "oztest"
    libdir = os.path.dirname(_lib.lib_path())
    subprocess.check_call(["g++", "-std=c++17", "-I", INCLUDE, os.path.join(ROOT, "example", "oztest.cpp"),
                           "-L", libdir, "-loz_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)])
    rc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert rc.returncode == (0 if HAVE_GPU else 2), rc.stderr


@pytest.mark.skipif(HAVE_GPU, reason="checks the no-device path")
def test_no_device_status_codes(ozlib):
    h = ozlib.Handle()
    assert h.setup(256, 512, 128, 0) == 2
    assert "device" in h.last_error().lower()
    C = np.zeros((4, 4))
    assert h.dgemm(4, 4, 4, np.ones((4, 4)), np.ones((4, 4)), C) != 0
    L = ozlib.load()
    assert L.ozgb_dgemm_device(h.raw, 4, 4, 4, None, 4, None, 4, None, 4, None) != 0
    h.close()


def test_option_validation(ozlib):
    L = ozlib.load()
    h = ozlib.Handle()
    assert L.ozgb_set_slices(h.raw, 41) == 7 and L.ozgb_set_slices(h.raw, 9) == 0
    assert L.ozgb_set_bits(h.raw, 8) == 7 and L.ozgb_set_bits(h.raw, 7) == 0
    assert L.ozgb_set_bins(h.raw, -2) == 7 and L.ozgb_set_bins(h.raw, -1) == 0
    assert L.ozgb_set_rounding(h.raw, 2) == 7 and L.ozgb_set_rounding(h.raw, 1) == 0
    assert L.ozgb_set_slice_format(h.raw, 2) == 7 and L.ozgb_set_slice_format(h.raw, 1) == 0
    assert L.ozgb_set_error_bound(h.raw, -1.0) == 7 and L.ozgb_set_error_bound(h.raw, 1e-15) == 0
    assert L.ozgb_set_profile(h.raw, 2) == 7 and L.ozgb_set_profile(h.raw, 1) == 0
    assert L.ozgb_set_timeout_ms(h.raw, 0.0) == 7
    assert L.ozgb_set_slices(None, 8) == 7
    h.close()


def _pairs(s, J):
    return sum(1 for p in range(s) for q in range(s) if p + q < J)


@pytest.mark.parametrize("shape", [(4096, 4096, 4096), (256, 512, 128), (1, 1, 1), (8192, 8192, 65536),
                                   (77, 91, 513), (2048, 32, 4096)])
@pytest.mark.parametrize("b,s,J", [(7, 8, 8), (7, 9, 9), (7, 8, 15), (3, 29, 29), (5, 11, 11), (7, 6, 6)])
def test_plan_invariants(ozlib, shape, b, s, J):
    """Every plan covers the bins with contiguous blocks of at most 256 TMEM
    columns, keeps each fp32 partial sum exact between drains, and has
    accumulator words for the largest exact sum."""
    M, N, K = shape
    c = ozlib.plan_query(M, N, K, b, s, J)
    assert c is not None
    assert (c["bits"], c["slices"], c["bins"]) == (b, s, J)
    assert c["pairs"] == _pairs(s, J)
    assert c["tile_n"] in (128, 64, 48, 32, 16)
    lo, nb = c["block_lo"], c["block_nb"]
    assert lo[0] == 0 and sum(nb) == J
    assert all(lo[g + 1] == lo[g] + nb[g] for g in range(len(lo) - 1))
    assert all(n * c["tile_n"] <= 256 for n in nb)
    max_pairs = max(_pairs(s, j + 1) - _pairs(s, j) for j in range(J))
    assert max_pairs * c["k_chunk"] * c["drain_chunks"] * (2 ** b - 1) ** 2 <= 2 ** 24
    qmax = sum((_pairs(s, j + 1) - _pairs(s, j)) * K * (2 ** b - 1) ** 2 << (b * (J - 1 - j)) for j in range(J))
    assert qmax.bit_length() + 1 <= 32 * c["acc_words"]
    # TMEM: one range per bin plus a second range for each double-buffered block
    dbl = c["dbl_blocks"]
    assert J * c["tile_n"] + sum(nb[g] * c["tile_n"] for g in range(c["blocks"]) if (dbl >> g) & 1) <= 512
    assert 1 <= c["issuers"] <= min(3, c["umma_per_kstep"])


@pytest.mark.parametrize("s,J,blocks", [(8, 9, [3, 3, 3]), (9, 9, [3, 3, 3]), (9, 10, [4, 3, 3])])
def test_partition_model_picks_the_measured_best(ozlib, s, J, blocks):
    """The planner's bin-block cost model picks, at BN = 48, the partition that
    was fastest among those timed on a GB300 at 4096^3 (sweeps over 6 to 15
    partitions per schedule), and the plan does not depend on K: its blocks, drain
    periods and issuers are the same for every K (the problems of a grouped call
    that share a shape class then share one launch)."""
    c = ozlib.plan_query(4096, 4096, 4096, 7, s, J)
    assert c["tile_n"] == 48 and c["block_nb"][:c["blocks"]] == blocks and c["issuers"] == 3
    for K in (32, 300, 4096, 65536):
        d = ozlib.plan_query(4096, 4096, K, 7, s, J)
        for key in ("tile_n", "blocks", "block_lo", "block_nb", "issuers", "dbl_blocks", "drain_chunks"):
            assert d[key] == c[key], (K, key)


def test_plan_rejects_inexact_requests(ozlib):
    assert ozlib.plan_query(128, 128, 128, 7, 30, 59) is None  # more than 8 bin blocks of TMEM
    assert ozlib.plan_query(0, 128, 128, 7, 8, 8) is None


def _stats(A, B):
    f = lambda x: ((x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int32)
    return (f(A).max(axis=1), (A * A).sum(axis=1), f(B).max(axis=0), (B * B).sum(axis=0), (A * A).sum(axis=0),
            (B * B).sum(axis=1))


def test_precision_knob_estimate_formula(ozlib, oracle):
    """The knob's estimate against a direct evaluation of its model:
    est(s) = 1.5 2^-bs ((s-1)/4 sqrt(K SA SB) + sqrt(SA |B|^2 / 3) + sqrt(SB |A|^2 / 3)) / sqrt(T) + 2^-53
    with SA = sum_i 4^(Er_i-1022), SB likewise, T = sum_k |A(:,k)|^2 |B(k,:)|^2."""
    K = 200
    A = oracle.gen_phi((64, K), 1, 1.0)
    B = oracle.gen_phi((K, 48), 2, 1.0)
    er, ssr, ec, ssc, ca, rb = _stats(A, B)
    SA = sum(4.0 ** (int(e) - 1022) for e in er)
    SB = sum(4.0 ** (int(e) - 1022) for e in ec)
    T = float(np.sum(ca * rb))
    nA, nB = float(ssr.sum()), float(ssc.sum())

    def model(t):
        return 1.5 * 2.0 ** (-7 * t) * ((t - 1) / 4 * (K * SA * SB) ** 0.5 + (SA * nB / 3) ** 0.5 +
                                        (SB * nA / 3) ** 0.5) / T ** 0.5 + 2.0 ** -53

    for bound in (1e-8, 1e-11, 1e-13, 1e-15):
        s, est = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, bound, ca, rb)
        assert est == pytest.approx(model(s), rel=1e-9)
        assert est <= bound and (s == 2 or model(s - 1) > bound)
    # without the k-direction sums the mass is taken as spread evenly over k
    s, est = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, 1e-15)
    assert 2 <= s <= 16 and est > 0


def test_precision_knob_degenerate_statistics(ozlib):
    """Zero, infinite or NaN statistics give the largest slice count, not a guess."""
    er = np.full(4, 1023, np.int32)
    ec = np.full(3, 1023, np.int32)
    for ss, ka in ((np.ones(4), np.zeros(8)), (np.full(4, np.inf), np.ones(8)), (np.full(4, np.nan), np.ones(8))):
        s, _ = ozlib.choose_slices(er, ss, ec, np.ones(3), 8, 7, 1e-15, ka, np.ones(8))
        assert s == 16


@pytest.mark.parametrize("phi", [0.1, 0.5, 1.0, 2.0, 4.0])
def test_precision_knob_meets_bound(ozlib, oracle, phi):
    """The slice count the knob picks from the stage-(a) statistics meets the
    requested normwise bound on the exact product (triangular pair set, RN)."""
    for (M, N, K), seed in (((96, 80, 300), 11), ((64, 64, 2048), 21)):
        A = oracle.gen_phi((M, K), seed, phi)
        B = oracle.gen_phi((K, N), seed + 1, phi)
        er, ssr, ec, ssc, ca, rb = _stats(A, B)
        rows = np.repeat(np.arange(M, dtype=np.int32), N)
        cols = np.tile(np.arange(N, dtype=np.int32), M)
        exact = oracle.exact_entries(A, B, rows, cols)[0].reshape(M, N)
        last = 0
        for bound in (1e-8, 1e-11, 1e-13, 1e-15):
            s, _ = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, bound, ca, rb)
            assert s >= last
            last = s
            C = oracle.dgemm(A, B, 7, s, s, 0)
            err = np.linalg.norm(C - exact) / np.linalg.norm(exact)
            assert err <= bound, (bound, s, err)


def test_version_string(ozlib):
    v = ozlib.load().ozgb_version()
    assert v and v.decode() if isinstance(v, bytes) else v


def test_reference_example_compiles_unchanged(ozlib, tmp_path):
    """The reference's own example program (example/oztest.cpp of Oz-AIE), where
    its sources are present, compiles and links against the drop-in header as is."""
    from oracle import build_oracle
    src = os.path.join(build_oracle.REFERENCE_ROOT, "example", "oztest.cpp")
    if not os.path.exists(src):
        pytest.skip("reference sources absent")
    from ozaie_gb300 import _lib
    libdir = os.path.dirname(_lib.lib_path())
    exe = tmp_path / "ref_oztest"
    subprocess.check_call(["g++", "-std=c++17", "-I", INCLUDE, src, "-L", libdir, "-loz_gb300",
                           "-Wl,-rpath," + libdir, "-o", str(exe)])
    rc = subprocess.run([str(exe)], capture_output=True, timeout=120)
    assert rc.returncode == (0 if HAVE_GPU else 2)


def test_cmake_use_ozaie_helper(ozlib, tmp_path):
    import shutil
    if not shutil.which("cmake"):
        pytest.skip("cmake absent")
    env = dict(os.environ, OZAIE_CMAKE_INCLUDE=os.path.join(INCLUDE, "CMakeLists.txt"))
    b = tmp_path / "b"
    subprocess.check_call(["cmake", "-S", os.path.join(ROOT, "example"), "-B", str(b)], env=env,
                          stdout=subprocess.DEVNULL)
    subprocess.check_call(["cmake", "--build", str(b)], env=env, stdout=subprocess.DEVNULL)
    rc = subprocess.run([str(b / "oztest")], capture_output=True, timeout=120)
    assert rc.returncode == (0 if HAVE_GPU else 2)


def test_tuning_table_starts_empty_and_clears(ozlib):
    from ozaie_gb300 import api
    api.tuning_clear()
    assert api.tuning_entries() == 0
    # a host-only plan query never consults or fills the table
    assert ozlib.plan_query(1024, 1024, 1024, 7, 9, 9) is not None
    assert api.tuning_entries() == 0


@pytest.mark.parametrize("b,s,J", [(4, 10, 10), (3, 18, 18), (4, 8, 15), (3, 29, 29), (2, 12, 12), (7, 9, 9)])
def test_plan_slice_format(ozlib, b, s, J):
    """Slices of b <= 4 bits plan on e4m3 (chunks of 32 or 64 K values), wider ones
    on bf16 (16 or 32); the fp32 exactness bound holds with the carrier's chunk."""
    M, N, K = 4096, 4096, 4096
    c = ozlib.plan_query(M, N, K, b, s, J)
    assert c is not None
    if b <= 4:
        assert c["slice_format"] == 1 and c["k_chunk"] in (32, 64)
    else:
        assert c["slice_format"] == 0 and c["k_chunk"] in (16, 32)
    max_pairs = max(_pairs(s, j + 1) - _pairs(s, j) for j in range(J))
    assert max_pairs * c["k_chunk"] * c["drain_chunks"] * (2 ** b - 1) ** 2 <= 2 ** 24


def test_precision_knob_elementwise_formula(ozlib, oracle):
    """The elementwise estimate against a direct evaluation of its model:
    est(s) = 4 2^-bs sqrt(K) sqrt(K (s-1)^2 ia ib / 16 + (ia + ib) / 3) / tail + 2^-53,
    ia = max_i 1 / (|a_i|^2 4^(1022 - Er_i)), ib likewise over the columns of B."""
    K = 300
    A = oracle.gen_phi((64, K), 3, 1.0)
    B = oracle.gen_phi((K, 48), 4, 1.0)
    er, ssr, ec, ssc, ca, rb = _stats(A, B)
    ia = max(1.0 / (float(x) * 4.0 ** (1022 - int(e))) for x, e in zip(ssr, er))
    ib = max(1.0 / (float(x) * 4.0 ** (1022 - int(e))) for x, e in zip(ssc, ec))
    for tail in (1e-2, 1e-4):
        def model(t):
            r = K * (t - 1) ** 2 * ia * ib / 16 + (ia + ib) / 3
            return 4.0 * 2.0 ** (-7 * t) * (K * r) ** 0.5 / tail + 2.0 ** -53

        for bound in (1e-8, 1e-11, 1e-15):
            s, est = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, bound, ca, rb, criterion=1, tail=tail)
            assert est == pytest.approx(model(s), rel=1e-9)
            assert est <= bound and (s == 2 or model(s - 1) > bound)
    # the elementwise criterion asks for at least as many slices as the normwise one
    sn, _ = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, 1e-13, ca, rb)
    se, _ = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, 1e-13, ca, rb, criterion=1, tail=1e-4)
    assert se >= sn
    assert ozlib.choose_slices(er, ssr, ec, ssc, K, 7, 1e-13, ca, rb, criterion=1, tail=0.0)[0] == -1


@pytest.mark.parametrize("phi", [0.5, 1.0, 2.0, 4.0])
def test_precision_knob_elementwise_meets_bound(ozlib, oracle, phi):
    """With the elementwise criterion, every entry at least tail |a_i| |b_j| /
    sqrt(K) away from zero meets the requested relative error against the exact
    product (triangular pair set, RN)."""
    tail = 1e-3
    M, N, K = 96, 80, 700
    A = oracle.gen_phi((M, K), 31, phi)
    B = oracle.gen_phi((K, N), 32, phi)
    er, ssr, ec, ssc, ca, rb = _stats(A, B)
    rows = np.repeat(np.arange(M, dtype=np.int32), N)
    cols = np.tile(np.arange(N, dtype=np.int32), M)
    exact = oracle.exact_entries(A, B, rows, cols)[0].reshape(M, N)
    scale = np.sqrt(np.outer(ssr, ssc) / K)
    kept = np.abs(exact) >= tail * scale
    assert kept.mean() > (0.99 if phi <= 2 else 0.8)
    for bound in (1e-8, 1e-11, 1e-13, 1e-15):
        s, _ = ozlib.choose_slices(er, ssr, ec, ssc, K, 7, bound, ca, rb, criterion=1, tail=tail)
        C = oracle.dgemm(A, B, 7, s, s, 0)
        rel = np.abs(C - exact)[kept] / np.abs(exact[kept])
        assert rel.max() <= bound, (bound, s, rel.max())


def test_grouped_launch_layout_walk(ozlib):
    """The grouped GEMM launches for the batched workload (512 problems, M, N, K
    log-uniform in [32, 2048]) and for ragged small shapes, walked on the host the
    way the kernel walks them: every tile of every problem once, every bulk copy
    inside its problem's slice blocks, the epilogue on its problem's C."""
    import bench
    sizes = [tuple(int(x) for x in r) for r in bench.batched_workload(512)]
    for s, J in ((9, 9), (8, 15), (4, 7), (12, 12)):
        rc, n_launch, units = ozlib.grouped_layout_check(sizes, s, J)
        assert rc == 0, (s, J, rc)
        # plans do not depend on K, so the 512 problems of one schedule share one launch
        assert n_launch == 1 and units > 512
    small = [(1, 1, 1), (129, 49, 17), (2048, 32, 2048), (32, 2048, 100), (300, 200, 500), (128, 48, 32)]
    rc, n_launch, units = ozlib.grouped_layout_check(small, 9, 9)
    assert rc == 0 and units >= len(small)


def test_precision_knob_pair_set_estimate_formula(ozlib, oracle):
    """The estimate of the pair set p + q <= J - 1 (s <= J <= 2s - 1): the first
    dropped pairs are the pairs_in_bin(J, s) pairs p + q = J of weight
    2^(-bJ)/4; the truncated tails stay at 2^(-bs).  J = s is the triangular
    formula; J = 2s - 1 (the full set) keeps the tails alone."""
    K = 200
    A = oracle.gen_phi((64, K), 5, 1.0)
    B = oracle.gen_phi((K, 48), 6, 1.0)
    er, ssr, ec, ssc, ca, rb = _stats(A, B)
    SA = sum(4.0 ** (int(e) - 1022) for e in er)
    SB = sum(4.0 ** (int(e) - 1022) for e in ec)
    T = float(np.sum(ca * rb))
    nA, nB = float(ssr.sum()), float(ssc.sum())

    def pairs(j, s):
        return max(0, min(j, s - 1) - max(0, j - (s - 1)) + 1)

    def model(s, J):
        nd = pairs(J, s) if J < 2 * s - 1 else 0
        return 1.5 * ((nd / 4) * 2.0 ** (-7 * J) * (K * SA * SB) ** 0.5 +
                      2.0 ** (-7 * s) * ((SA * nB / 3) ** 0.5 + (SB * nA / 3) ** 0.5)) / T ** 0.5 + 2.0 ** -53

    for bound in (1e-8, 1e-11, 1e-13, 1e-15):
        s, J, est = ozlib.choose_schedule(er, ssr, ec, ssc, K, 7, bound, ca, rb)
        assert s <= J <= 2 * s - 1
        assert est == pytest.approx(model(s, J), rel=1e-9) and est <= bound
        # the triangular search agrees with the slice-only knob
        st, Jt, _ = ozlib.choose_schedule(er, ssr, ec, ssc, K, 7, bound, ca, rb, any_pair_set=0)
        assert Jt == st == ozlib.choose_slices(er, ssr, ec, ssc, K, 7, bound, ca, rb)[0]


@pytest.mark.parametrize("phi", [0.5, 1.0, 2.0, 4.0])
def test_slice_schedule_meets_bound(ozlib, oracle, phi):
    """The slice schedule (s, J) the knob picks when it searches every pair set
    meets the requested normwise bound on the exact product, and with the
    elementwise criterion the elementwise bound on every entry at least
    tail |a_i| |b_j| / sqrt(K) from zero."""
    tail = 1e-3
    for (M, N, K), seed in (((96, 80, 300), 13), ((64, 64, 2048), 23)):
        A = oracle.gen_phi((M, K), seed, phi)
        B = oracle.gen_phi((K, N), seed + 1, phi)
        er, ssr, ec, ssc, ca, rb = _stats(A, B)
        rows = np.repeat(np.arange(M, dtype=np.int32), N)
        cols = np.tile(np.arange(N, dtype=np.int32), M)
        exact = oracle.exact_entries(A, B, rows, cols)[0].reshape(M, N)
        kept = np.abs(exact) >= tail * np.sqrt(np.outer(ssr, ssc) / K)
        for bound in (1e-8, 1e-11, 1e-13, 1e-15):
            s, J, _ = ozlib.choose_schedule(er, ssr, ec, ssc, K, 7, bound, ca, rb)
            C = oracle.dgemm(A, B, 7, s, J, 0)
            err = np.linalg.norm(C - exact) / np.linalg.norm(exact)
            assert err <= bound, (bound, s, J, err)
            s, J, _ = ozlib.choose_schedule(er, ssr, ec, ssc, K, 7, bound, ca, rb, criterion=1, tail=tail)
            C = oracle.dgemm(A, B, 7, s, J, 0)
            rel = np.abs(C - exact)[kept] / np.abs(exact[kept])
            assert rel.max() <= bound, (bound, s, J, rel.max())


def test_slice_schedule_prefers_fewer_umma(ozlib):
    """At 4096^3 with phi = 1 statistics and a 1e-15 normwise bound, the search
    takes 8 slices with the pair set p + q <= 8 (13 UMMAs per 16-deep K step of a
    128 x 48 tile) over the triangular 9 slices (14): same bound, less work."""
    from oracle import ozoracle as O
    A = O.gen_phi((4096, 4096), 1, 1.0)
    B = O.gen_phi((4096, 4096), 2, 1.0)
    er, ssr, ec, ssc, ca, rb = _stats(A, B)
    s, J, est = ozlib.choose_schedule(er, ssr, ec, ssc, 4096, 7, 1e-15, ca, rb)
    st, Jt, _ = ozlib.choose_schedule(er, ssr, ec, ssc, 4096, 7, 1e-15, ca, rb, any_pair_set=0)
    assert (st, Jt) == (9, 9) and (s, J) == (8, 9) and est <= 1e-15
    a = ozlib.plan_query(4096, 4096, 4096, 7, s, J)
    b = ozlib.plan_query(4096, 4096, 4096, 7, st, Jt)
    assert a["umma_per_kstep"] / a["tile_n"] < b["umma_per_kstep"] / b["tile_n"]
