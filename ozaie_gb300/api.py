"""Python mirror of the Oz-AIE API over the GB300 C ABI.

Same names, argument meaning and status codes as the reference's C++ API
(atlarge-research/ozAIE include/oz_aie.h):
    Mode.accurate / Mode.fast                       (:82)
    ozAIE_setup(M, N, K, mode) -> int status        (:182-300)
    ozAIE_DGEMM(M, N, K, A, B, C) -> int status     (:311-349), C overwritten with A @ B
    convert_paired_i64_to_double_matrix(...)        (:92-150)
    cleanup_xrt()                                   (:153-170)
A, B, C are row-major float64 numpy arrays (host memory), as the reference's
host double arrays.  The module-level functions use one default handle, like
the reference's process-global state; `Handle` is the explicit, thread-safe form.
"""
import ctypes
import enum

import numpy as np

from ._lib import OzgbConfig, OzgbError, OzgbProblem, load


class Mode(enum.IntEnum):
    accurate = 0
    fast = 1


class Profile(enum.IntEnum):
    gb300 = 0
    reference = 1


class Criterion(enum.IntEnum):
    normwise = 0
    elementwise = 1


class Rounding(enum.IntEnum):
    default = -1
    nearest = 0
    reference = 1


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Handle:
    """One library context (device buffers, options, stream)."""

    def __init__(self):
        self._L = load()
        h = ctypes.c_void_p()
        rc = self._L.ozgb_create(ctypes.byref(h))
        if rc:
            raise OzgbError(rc, "ozgb_create failed")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.ozgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ helpers
    @property
    def raw(self):
        return self._h

    def last_error(self):
        return self._L.ozgb_last_error(self._h).decode()

    def _check(self, rc):
        if rc:
            raise OzgbError(rc, self.last_error())
        return rc

    # ----------------------------------------------------------- drop-in
    def setup(self, M, N, K, mode=Mode.accurate):
        return self._L.ozgb_setup(self._h, int(M), int(N), int(K), int(mode))

    def dgemm(self, M, N, K, A, B, C):
        for name, arr, shape in (("A", A, (M, K)), ("B", B, (K, N)), ("C", C, (M, N))):
            if arr.dtype != np.float64 or not arr.flags.c_contiguous or arr.size != shape[0] * shape[1]:
                raise ValueError("%s must be a C-contiguous float64 array with %d elements" % (name, shape[0] * shape[1]))
        if not C.flags.writeable:
            raise ValueError("C must be writeable")
        return self._L.ozgb_dgemm(self._h, int(M), int(N), int(K), _ptr(A), _ptr(B), _ptr(C))

    def matmul(self, A, B, mode=None):
        """Convenience: returns A @ B (setup + DGEMM), raising on error."""
        A = np.ascontiguousarray(A, np.float64)
        B = np.ascontiguousarray(B, np.float64)
        M, K = A.shape
        N = B.shape[1]
        self._check(self.setup(M, N, K, Mode.fast if mode is None else mode))
        C = np.empty((M, N), np.float64)
        self._check(self.dgemm(M, N, K, A, B, C))
        return C

    # ---------------------------------------------------- device pointers
    def dgemm_device(self, M, N, K, dA, lda, dB, ldb, dC, ldc, stream=None):
        return self._L.ozgb_dgemm_device(self._h, M, N, K, ctypes.c_void_p(dA), lda, ctypes.c_void_p(dB), ldb,
                                         ctypes.c_void_p(dC), ldc, ctypes.c_void_p(stream or 0))

    def dgemm_ex(self, transa, transb, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc, stream=None):
        """C = alpha op(A) op(B) + beta C on device pointers (row-major, BLAS-style)."""
        return self._L.ozgb_dgemm_ex(self._h, int(transa), int(transb), M, N, K, float(alpha), dA, lda, dB, ldb,
                                     float(beta), dC, ldc, ctypes.c_void_p(stream or 0))

    def dgemm_grouped(self, problems, stream=None, with_bins=False):
        """Returns (status, slices used per problem), or with with_bins (status,
        [(slices, bins)] per problem)."""
        arr = (OzgbProblem * len(problems))()
        for i, p in enumerate(problems):
            arr[i] = OzgbProblem(p["M"], p["N"], p["K"], p["A"], p["lda"], p["B"], p["ldb"], p["C"], p["ldc"],
                                 float(p.get("error_bound", 0.0)), 0, 0)
        rc = self._L.ozgb_dgemm_grouped(self._h, arr, len(problems), ctypes.c_void_p(stream or 0))
        if with_bins:
            return rc, [(arr[i].slices_used, arr[i].bins_used) for i in range(len(problems))]
        return rc, [arr[i].slices_used for i in range(len(problems))]

    def sync(self):
        return self._L.ozgb_sync(self._h)

    # ------------------------------------------------------------- options
    def set_profile(self, p):
        return self._check(self._L.ozgb_set_profile(self._h, int(p)))

    def set_bits(self, b):
        return self._check(self._L.ozgb_set_bits(self._h, int(b)))

    def set_slices(self, s):
        return self._check(self._L.ozgb_set_slices(self._h, int(s)))

    def set_bins(self, j):
        return self._check(self._L.ozgb_set_bins(self._h, int(j)))

    def set_rounding(self, r):
        return self._check(self._L.ozgb_set_rounding(self._h, int(r)))

    def set_plan_hint(self, tile_n=0, k_chunk=0, stages=0, issuers=0, dbl=-1, block_nb=()):
        """Fix choices of the slice-pair GEMM plan (0 / -1 / () = the planner's)."""
        arr = (ctypes.c_int * max(1, len(block_nb)))(*block_nb) if block_nb else None
        return self._check(self._L.ozgb_set_plan_hint(self._h, int(tile_n), int(k_chunk), int(stages),
                                                      int(issuers), int(dbl), len(block_nb),
                                                      ctypes.cast(arr, ctypes.c_void_p) if arr else None))

    def set_slice_format(self, fmt):
        """0: e4m3 slices where exact (b <= 4), else bf16; 1: bf16 always."""
        return self._check(self._L.ozgb_set_slice_format(self._h, int(fmt)))

    def set_error_bound(self, e):
        return self._check(self._L.ozgb_set_error_bound(self._h, float(e)))

    def set_error_criterion(self, criterion, tail=1e-4):
        """Criterion.normwise (default) or Criterion.elementwise with its tail."""
        return self._check(self._L.ozgb_set_error_criterion(self._h, int(criterion), float(tail)))

    def set_graph(self, on):
        return self._check(self._L.ozgb_set_graph(self._h, 1 if on else 0))

    def set_schedule_search(self, any_pair_set):
        """1: the knob searches every pair set (default); 0: the triangular set only."""
        return self._check(self._L.ozgb_set_schedule_search(self._h, int(any_pair_set)))

    def set_grouped_launch(self, mode):
        """1: one persistent GEMM launch per plan class (default); 0: one per problem."""
        return self._check(self._L.ozgb_set_grouped_launch(self._h, int(mode)))

    def set_timeout_ms(self, ms):
        return self._check(self._L.ozgb_set_timeout_ms(self._h, float(ms)))

    def set_profiling(self, on):
        return self._check(self._L.ozgb_set_profiling(self._h, 1 if on else 0))

    def stage_times(self):
        t = (ctypes.c_float * 4)()
        self._check(self._L.ozgb_stage_times(self._h, t, 4))
        return {"exponents": t[0], "split": t[1], "gemm": t[2], "total": t[3]}

    def autotune(self, M, N, K, bits=7, slices=9, bins=0, max_candidates=64):
        """Times candidate plans for this configuration and records the fastest
        in the process-wide tuning table; returns its configuration."""
        c = OzgbConfig()
        self._check(self._L.ozgb_autotune(self._h, M, N, K, bits, slices, bins, max_candidates, ctypes.byref(c)))
        return c.as_dict()

    def launch_count(self):
        n = ctypes.c_longlong()
        self._check(self._L.ozgb_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def config(self):
        c = OzgbConfig()
        self._check(self._L.ozgb_get_config(self._h, ctypes.byref(c)))
        return c.as_dict()

    # -------------------------------------------------------- test hooks
    def dump(self, A, B, bin_lo=0, bin_hi=63, want_slices=True, want_q=True):
        """Intermediates for parity checks: er, ec, A/B int8 slice planes, q words."""
        A = np.ascontiguousarray(A, np.float64)
        B = np.ascontiguousarray(B, np.float64)
        M, K = A.shape
        N = B.shape[1]
        er = np.zeros(M, np.int32)
        ec = np.zeros(N, np.int32)
        s_max = 40
        asl = np.zeros((s_max, M, K), np.int8) if want_slices else None
        bsl = np.zeros((s_max, K, N), np.int8) if want_slices else None
        q = np.zeros((M, N, 4), np.int32) if want_q else None
        rc = self._L.ozgb_dump(self._h, M, N, K, _ptr(A), _ptr(B), _ptr(er), _ptr(ec),
                               _ptr(asl) if want_slices else None, _ptr(bsl) if want_slices else None,
                               _ptr(q) if want_q else None, int(bin_lo), int(bin_hi))
        self._check(rc)
        s = self.config()["slices"]
        out = {"er": er, "ec": ec, "config": self.config()}
        if want_slices:
            out["a_slices"] = asl[:s]
            out["b_slices"] = bsl[:s]
        if want_q:
            out["q"] = q
        return out

    def dump_pairs(self, A, B):
        """The reference's device output (int64 lo, hi per element, shape [M, N, 2])."""
        A = np.ascontiguousarray(A, np.float64)
        B = np.ascontiguousarray(B, np.float64)
        M, K = A.shape
        N = B.shape[1]
        out = np.zeros((M, N, 2), np.int64)
        self._check(self._L.ozgb_dump_pairs(self._h, M, N, K, _ptr(A), _ptr(B), _ptr(out)))
        return out

    def selftest_timeout(self, ms):
        return self._L.ozgb_selftest_timeout(self._h, float(ms))


def q_words_to_int(q):
    """int32[..., 4] little-endian two's complement words -> Python ints (object array)."""
    q = np.asarray(q).astype(np.int64) & 0xFFFFFFFF
    flat = q.reshape(-1, 4)
    out = np.empty(flat.shape[0], dtype=object)
    for i, w in enumerate(flat):
        v = int(w[0]) | (int(w[1]) << 32) | (int(w[2]) << 64) | (int(w[3]) << 96)
        if v >= 1 << 127:
            v -= 1 << 128
        out[i] = v
    return out.reshape(q.shape[:-1])


def tuning_entries():
    return load().ozgb_tuning_entries()


def tuning_clear():
    load().ozgb_tuning_clear()


def grouped_layout_check(sizes, slices, bins=0):
    """Host-only walk of the grouped launches for problems of the given (M, N, K)
    sizes: (status, launches, work units); status 0 when every check holds."""
    arr = (OzgbProblem * len(sizes))()
    base = 1 << 42
    for i, (M, N, K) in enumerate(sizes):
        arr[i] = OzgbProblem(int(M), int(N), int(K), None, int(K), None, int(N), base, int(N), 0.0, 0, 0)
        base += ((int(M) * int(N) * 8 + 255) // 256) * 256
    nl = ctypes.c_int()
    nu = ctypes.c_longlong()
    rc = load().ozgb_grouped_layout_check(arr, len(sizes), int(slices), int(bins), ctypes.byref(nl), ctypes.byref(nu))
    return rc, nl.value, nu.value


def plan_query(M, N, K, bits, slices, bins):
    c = OzgbConfig()
    rc = load().ozgb_plan_query(M, N, K, bits, slices, bins, ctypes.byref(c))
    return None if rc else c.as_dict()


def choose_slices(er, ssr, ec, ssc, K, bits, bound, sa_k=None, sb_k=None, criterion=0, tail=1e-4):
    """Host-only precision knob: (slice count, a-priori error estimate) for a
    requested bound, from the stage-(a) statistics.  sa_k / sb_k are the sums of
    squares of the columns of A and the rows of B (None: spread evenly);
    criterion 0 bounds the normwise error, 1 the elementwise error of the
    entries at least tail sigma_ij away from zero."""
    er = np.ascontiguousarray(er, np.int32)
    ec = np.ascontiguousarray(ec, np.int32)
    ssr = np.ascontiguousarray(ssr, np.float64)
    ssc = np.ascontiguousarray(ssc, np.float64)
    ka = None if sa_k is None else np.ascontiguousarray(sa_k, np.float64)
    kb = None if sb_k is None else np.ascontiguousarray(sb_k, np.float64)
    est = ctypes.c_double()
    s = load().ozgb_choose_slices_ex(_ptr(er), _ptr(ssr), er.size, _ptr(ec), _ptr(ssc), ec.size,
                                     None if ka is None else _ptr(ka), None if kb is None else _ptr(kb), int(K),
                                     int(bits), float(bound), int(criterion), float(tail), ctypes.byref(est))
    return s, est.value


def choose_schedule(er, ssr, ec, ssc, K, bits, bound, sa_k=None, sb_k=None, criterion=0, tail=1e-4,
                    any_pair_set=1, sms=152):
    """Host-only slice schedule: (slices, bins, estimate) that the knob picks for
    these stage-(a) statistics (M = len(er), N = len(ec)) on a device with `sms` SMs."""
    er = np.ascontiguousarray(er, np.int32)
    ec = np.ascontiguousarray(ec, np.int32)
    ssr = np.ascontiguousarray(ssr, np.float64)
    ssc = np.ascontiguousarray(ssc, np.float64)
    ka = None if sa_k is None else np.ascontiguousarray(sa_k, np.float64)
    kb = None if sb_k is None else np.ascontiguousarray(sb_k, np.float64)
    s, J, est = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    rc = load().ozgb_choose_schedule(_ptr(er), _ptr(ssr), er.size, _ptr(ec), _ptr(ssc), ec.size,
                                     None if ka is None else _ptr(ka), None if kb is None else _ptr(kb), int(K),
                                     int(bits), float(bound), int(criterion), float(tail), int(any_pair_set), int(sms),
                                     ctypes.byref(s), ctypes.byref(J), ctypes.byref(est))
    if rc:
        raise ValueError("ozgb_choose_schedule: bad input")
    return s.value, J.value, est.value


def convert_paired_i64_to_double_matrix(C, result, M, N, K, num_splits, bits_per_slice):
    """include/oz_aie.h:92-150 on numpy arrays (C: int64[M*N*2], result: float64[M*N])."""
    C = np.ascontiguousarray(C, np.int64)
    rc = load().ozgb_convert_paired_i64_to_double(_ptr(C), _ptr(result), M, N, K, num_splits, bits_per_slice)
    if rc:
        raise OzgbError(rc, "bad arguments")


# ----------------------------------------------- process-global default
_default = None


def _handle():
    global _default
    if _default is None:
        _default = Handle()
    return _default


def ozAIE_setup(M, N, K, mode):
    return _handle().setup(M, N, K, mode)


def ozAIE_DGEMM(M, N, K, A, B, C):
    return _handle().dgemm(M, N, K, A, B, C)


def cleanup_xrt():
    if _default is not None:
        load().ozgb_release(_default.raw)
