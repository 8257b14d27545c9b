"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  It wraps oracle/liboz_oracle.so (the CPU restatement of the reference's
Ozaki arithmetic) and, when built, oracle/_ref/libref_decode.so (the reference's
own host decode, compiled from its sources).
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None
_ref = None

_d = ctypes.POINTER(ctypes.c_double)
_i32 = ctypes.POINTER(ctypes.c_int32)
_i64 = ctypes.POINTER(ctypes.c_int64)
_i8 = ctypes.POINTER(ctypes.c_int8)
_int = ctypes.c_int


def _p(a, t):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.ORACLE_SO
        if not os.path.exists(path):
            build_oracle.build_oracle()
        L = ctypes.CDLL(path)
        L.ozo_max_exp_rows.argtypes = [_d, _int, _int, _i32]
        L.ozo_max_exp_cols.argtypes = [_d, _int, _int, _i32]
        L.ozo_split_elem.argtypes = [ctypes.c_uint64, _int, _int, _int, _i8, ctypes.c_long]
        L.ozo_split_rows.argtypes = [_d, _int, _int, _i32, _int, _int, _i8]
        L.ozo_split_cols.argtypes = [_d, _int, _int, _i32, _int, _int, _i8]
        L.ozo_bins.argtypes = [_i8, _i8, _int, _int, _int, _int, _int, _i64]
        L.ozo_sum_upshift.argtypes = [_i64, _i32, _i32, _int, _int, _int, _int, _int, _i64]
        L.ozo_first_group.argtypes = [_int, _int, _int]
        L.ozo_first_group.restype = _int
        L.ozo_decode_pairs.argtypes = [_i64, _d, _int, _int, _int, _int, _int]
        L.ozo_finish.argtypes = [_i64, _i32, _i32, _int, _int, _int, _int, _int, _d, ctypes.c_void_p]
        L.ozo_dgemm.argtypes = [_d, _d, _d, _int, _int, _int, _int, _int, _int, _int]
        L.ozo_dgemm_rows.argtypes = [_d, _d, _d, _int, _int, _int, _int, _int, _int, _int, _int, _int]
        L.ozo_exact_entries.argtypes = [_d, _d, _int, _int, _int, _i32, _i32, _int, _d, ctypes.c_void_p]
        L.ozo_mpfr_entries.argtypes = [_d, _d, _int, _int, _int, _i32, _i32, _int, _int, _d]
        L.ozo_mpfr_entries.restype = _int
        L.ozo_dgemm_naive.argtypes = [_d, _d, _d, _int, _int, _int]
        L.ozo_num_threads.restype = _int
        _lib = L
    return _lib


def ref_decode_lib():
    """The reference's compiled decode, or None when the reference is absent."""
    global _ref
    if _ref is None:
        path = build_oracle.REF_SO
        if not os.path.exists(path):
            if build_oracle.build_ref_decode() is None:
                return None
        R = ctypes.CDLL(path)
        R.ref_convert_paired_i64_to_double_matrix.argtypes = [_i64, _d, _int, _int, _int, _int, _int]
        _ref = R
    return _ref


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def max_exp_rows(A):
    A = _c(A, np.float64)
    M, K = A.shape
    out = np.zeros(M, np.int32)
    lib().ozo_max_exp_rows(_p(A, _d), M, K, _p(out, _i32))
    return out


def max_exp_cols(B):
    B = _c(B, np.float64)
    K, N = B.shape
    out = np.zeros(N, np.int32)
    lib().ozo_max_exp_cols(_p(B, _d), K, N, _p(out, _i32))
    return out


def split_rows(A, Er, b, d):
    A = _c(A, np.float64)
    Er = _c(Er, np.int32)
    M, K = A.shape
    out = np.zeros((d, M, K), np.int8)
    lib().ozo_split_rows(_p(A, _d), M, K, _p(Er, _i32), b, d, _p(out, _i8))
    return out


def split_cols(B, Ec, b, d):
    B = _c(B, np.float64)
    Ec = _c(Ec, np.int32)
    K, N = B.shape
    out = np.zeros((d, K, N), np.int8)
    lib().ozo_split_cols(_p(B, _d), K, N, _p(Ec, _i32), b, d, _p(out, _i8))
    return out


def split_values(x, E, b, d):
    """Slices of each double in x (1-D) against the matching exponent in E."""
    x = _c(x, np.float64).ravel()
    E = np.broadcast_to(np.asarray(E, np.int32), x.shape)
    out = np.zeros((x.size, d), np.int8)
    L = lib()
    for i, (v, e) in enumerate(zip(x.view(np.uint64), E)):
        L.ozo_split_elem(int(v), int(e), b, d, out[i].ctypes.data_as(_i8), 1)
    return out


def bins(Ap, Bp, J):
    Ap = _c(Ap, np.int8)
    Bp = _c(Bp, np.int8)
    d, M, K = Ap.shape
    d2, K2, N = Bp.shape
    assert d == d2 and K == K2
    out = np.zeros((J, M, N), np.int64)
    lib().ozo_bins(_p(Ap, _i8), _p(Bp, _i8), M, N, K, d, J, _p(out, _i64))
    return out


def first_group(K, b, d):
    return lib().ozo_first_group(K, b, d)


def sum_upshift(bins_, Er, Ec, K, b, d):
    bins_ = _c(bins_, np.int64)
    J, M, N = bins_.shape
    assert J >= d
    out = np.zeros((M, N, 2), np.int64)
    lib().ozo_sum_upshift(_p(bins_, _i64), _p(_c(Er, np.int32), _i32), _p(_c(Ec, np.int32), _i32),
                          M, N, K, b, d, _p(out, _i64))
    return out


def decode_pairs(pairs, K, d, b):
    pairs = _c(pairs, np.int64)
    M, N, _ = pairs.shape
    out = np.zeros((M, N), np.float64)
    lib().ozo_decode_pairs(_p(pairs, _i64), _p(out, _d), M, N, K, d, b)
    return out


def ref_decode_pairs(pairs, K, d, b):
    """The reference's own decode (compiled from its header); None if unavailable."""
    R = ref_decode_lib()
    if R is None:
        return None
    pairs = np.array(pairs, dtype=np.int64, copy=True, order="C")
    M, N, _ = pairs.shape
    out = np.zeros((M, N), np.float64)
    R.ref_convert_paired_i64_to_double_matrix(_p(pairs, _i64), _p(out, _d), M, N, K, d, b)
    return out


def finish(bins_, Er, Ec, b, rounding=0, want_q=False):
    bins_ = _c(bins_, np.int64)
    J, M, N = bins_.shape
    C = np.zeros((M, N), np.float64)
    q = np.zeros((M, N, 4), np.int64) if want_q else None
    lib().ozo_finish(_p(bins_, _i64), _p(_c(Er, np.int32), _i32), _p(_c(Ec, np.int32), _i32),
                     M, N, b, J, rounding, _p(C, _d), q.ctypes.data if want_q else None)
    return (C, q) if want_q else C


def dgemm(A, B, b, d, J=None, rounding=0):
    A = _c(A, np.float64)
    B = _c(B, np.float64)
    M, K = A.shape
    K2, N = B.shape
    assert K == K2
    C = np.zeros((M, N), np.float64)
    lib().ozo_dgemm(_p(A, _d), _p(B, _d), _p(C, _d), M, N, K, b, d, d if J is None else J, rounding)
    return C


def dgemm_rows(A, B, b, d, J, rounding, r0, r1):
    """Oracle pipeline on rows [r0, r1) of A only; returns C[r0:r1]."""
    A = _c(A, np.float64)
    B = _c(B, np.float64)
    M, K = A.shape
    N = B.shape[1]
    C = np.zeros((M, N), np.float64)
    lib().ozo_dgemm_rows(_p(A, _d), _p(B, _d), _p(C, _d), M, N, K, b, d, J, rounding, r0, r1)
    return C[r0:r1]


def exact_entries(A, B, rows, cols):
    A = _c(A, np.float64)
    B = _c(B, np.float64)
    rows = _c(rows, np.int32)
    cols = _c(cols, np.int32)
    M, K = A.shape
    N = B.shape[1]
    out = np.zeros(rows.size, np.float64)
    absdot = np.zeros(rows.size, np.float64)
    lib().ozo_exact_entries(_p(A, _d), _p(B, _d), M, N, K, _p(rows, _i32), _p(cols, _i32), rows.size,
                            _p(out, _d), absdot.ctypes.data)
    return out, absdot


def mpfr_entries(A, B, rows, cols, prec=106):
    """MPFR mirror of mul_acc_MPFR; None when libmpfr.so.6 cannot be loaded."""
    A = _c(A, np.float64)
    B = _c(B, np.float64)
    rows = _c(rows, np.int32)
    cols = _c(cols, np.int32)
    M, K = A.shape
    N = B.shape[1]
    out = np.zeros(rows.size, np.float64)
    rc = lib().ozo_mpfr_entries(_p(A, _d), _p(B, _d), M, N, K, _p(rows, _i32), _p(cols, _i32), rows.size,
                                prec, _p(out, _d))
    return None if rc != 0 else out


def dgemm_naive(A, B):
    A = _c(A, np.float64)
    B = _c(B, np.float64)
    M, K = A.shape
    N = B.shape[1]
    C = np.zeros((M, N), np.float64)
    lib().ozo_dgemm_naive(_p(A, _d), _p(B, _d), _p(C, _d), M, N, K)
    return C


def num_threads():
    return lib().ozo_num_threads()


# ----------------------------------------------------------- test matrices
def gen_uniform(shape, seed, lo=-1.0, hi=1.0):
    return np.random.default_rng(seed).uniform(lo, hi, size=shape)


def gen_phi(shape, seed, phi):
    """a_ij = (U(0,1) - 0.5) * exp(phi * N(0,1)), the reference harness's family
    (test.cpp:219-237), drawn with numpy's PCG64 generator."""
    g = np.random.default_rng(seed)
    u = g.random(shape) - 0.5
    n = g.standard_normal(shape)
    return u * np.exp(phi * n)


def sample_indices(M, N, n, seed=0):
    g = np.random.default_rng(seed)
    return g.integers(0, M, n).astype(np.int32), g.integers(0, N, n).astype(np.int32)


def error_report(C, A, B, rows, cols, Cexact=None, absdot=None):
    """Errors of C at the sampled entries against the exact products."""
    if Cexact is None:
        Cexact, absdot = exact_entries(A, B, rows, cols)
    c = np.asarray(C)[rows, cols]
    diff = np.abs(c - Cexact)
    nrm = np.linalg.norm(Cexact)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(Cexact != 0, diff / np.abs(Cexact), np.where(diff == 0, 0.0, np.inf))
        comp = np.where(absdot != 0, diff / absdot, np.where(diff == 0, 0.0, np.inf))
    return {
        "normwise_rel": float(np.linalg.norm(c - Cexact) / nrm) if nrm > 0 else float(np.linalg.norm(c)),
        "max_rel": float(np.max(rel)) if rel.size else 0.0,
        "median_rel": float(np.median(rel)) if rel.size else 0.0,
        "max_componentwise": float(np.max(comp)) if comp.size else 0.0,
    }
