"""ctypes binding of liboz_gb300.so (the C ABI declared in include/oz_gb300.h).

The shared library is built in-tree by ozaie_gb300.build.  There is no CPU
fallback: if the library is missing, loading raises, and every compute entry
point returns OZGB_ERR_NO_DEVICE when no CUDA device is present.
"""
import ctypes
import os

from . import build as _build

_lib = None


class OzgbConfig(ctypes.Structure):
    _fields_ = [
        ("bits", ctypes.c_int),
        ("slices", ctypes.c_int),
        ("bins", ctypes.c_int),
        ("rounding", ctypes.c_int),
        ("tile_n", ctypes.c_int),
        ("k_chunk", ctypes.c_int),
        ("stages", ctypes.c_int),
        ("drain_chunks", ctypes.c_int),
        ("acc_words", ctypes.c_int),
        ("pairs", ctypes.c_int),
        ("blocks", ctypes.c_int),
        ("umma_per_kstep", ctypes.c_int),
        ("block_lo", ctypes.c_int * 8),
        ("block_nb", ctypes.c_int * 8),
        ("issuers", ctypes.c_int),
        ("slice_format", ctypes.c_int),
        ("dbl_blocks", ctypes.c_int),
    ]

    def as_dict(self):
        d = {}
        for f, _ in self._fields_:
            v = getattr(self, f)
            d[f] = list(v)[: self.blocks] if f in ("block_lo", "block_nb") else v
        return d


class OzgbProblem(ctypes.Structure):
    _fields_ = [
        ("M", ctypes.c_int), ("N", ctypes.c_int), ("K", ctypes.c_int),
        ("A", ctypes.c_void_p), ("lda", ctypes.c_long),
        ("B", ctypes.c_void_p), ("ldb", ctypes.c_long),
        ("C", ctypes.c_void_p), ("ldc", ctypes.c_long),
        ("error_bound", ctypes.c_double),
        ("slices_used", ctypes.c_int),
        ("bins_used", ctypes.c_int),
    ]


STATUS = {
    0: "OZGB_OK", 1: "OZGB_ERR_DIMS", 2: "OZGB_ERR_NO_DEVICE", 3: "OZGB_ERR_EXEC", 4: "OZGB_ERR_IMAGE",
    5: "OZGB_ERR_NOT_SETUP", 6: "OZGB_ERR_DIM_MISMATCH", 7: "OZGB_ERR_ARG", 8: "OZGB_ERR_ALLOC",
    9: "OZGB_ERR_TIMEOUT", 10: "OZGB_ERR_UNSUPPORTED", 11: "OZGB_ERR_TOO_LARGE",
}

# (name, restype, argtypes) for every function of include/oz_gb300.h
_h = ctypes.c_void_p
_i = ctypes.c_int
_l = ctypes.c_long
_p = ctypes.c_void_p
_dbl = ctypes.c_double
SIGNATURES = [
    ("ozgb_create", _i, [ctypes.POINTER(_h)]),
    ("ozgb_destroy", _i, [_h]),
    ("ozgb_release", _i, [_h]),
    ("ozgb_setup", _i, [_h, _i, _i, _i, _i]),
    ("ozgb_dgemm", _i, [_h, _i, _i, _i, _p, _p, _p]),
    ("ozgb_dgemm_device", _i, [_h, _i, _i, _i, _p, _l, _p, _l, _p, _l, _p]),
    ("ozgb_sync", _i, [_h]),
    ("ozgb_dgemm_grouped", _i, [_h, ctypes.POINTER(OzgbProblem), _i, _p]),
    ("ozgb_set_profile", _i, [_h, _i]),
    ("ozgb_set_bits", _i, [_h, _i]),
    ("ozgb_set_slices", _i, [_h, _i]),
    ("ozgb_set_bins", _i, [_h, _i]),
    ("ozgb_set_rounding", _i, [_h, _i]),
    ("ozgb_set_slice_format", _i, [_h, _i]),
    ("ozgb_set_plan_hint", _i, [_h, _i, _i, _i, _i, _i, _i, ctypes.c_void_p]),
    ("ozgb_set_error_bound", _i, [_h, _dbl]),
    ("ozgb_set_error_criterion", _i, [_h, _i, _dbl]),
    ("ozgb_set_graph", _i, [_h, _i]),
    ("ozgb_set_grouped_launch", _i, [_h, _i]),
    ("ozgb_set_schedule_search", _i, [_h, _i]),
    ("ozgb_choose_schedule", _i, [_p, _p, _i, _p, _p, _i, _p, _p, _i, _i, _dbl, _i, _dbl, _i, _i,
                                  ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_dbl)]),
    ("ozgb_grouped_layout_check", _i, [ctypes.POINTER(OzgbProblem), _i, _i, _i, ctypes.POINTER(_i),
                                       ctypes.POINTER(ctypes.c_longlong)]),
    ("ozgb_set_timeout_ms", _i, [_h, _dbl]),
    ("ozgb_get_config", _i, [_h, ctypes.POINTER(OzgbConfig)]),
    ("ozgb_set_profiling", _i, [_h, _i]),
    ("ozgb_stage_times", _i, [_h, ctypes.POINTER(ctypes.c_float), _i]),
    ("ozgb_last_error", ctypes.c_char_p, [_h]),
    ("ozgb_dump", _i, [_h, _i, _i, _i, _p, _p, _p, _p, _p, _p, _p, _i, _i]),
    ("ozgb_selftest_timeout", _i, [_h, _dbl]),
    ("ozgb_convert_paired_i64_to_double", _i, [_p, _p, _i, _i, _i, _i, _i]),
    ("ozgb_plan_query", _i, [_i, _i, _i, _i, _i, _i, ctypes.POINTER(OzgbConfig)]),
    ("ozgb_choose_slices", _i, [_p, _p, _i, _p, _p, _i, _p, _p, _i, _i, _dbl, ctypes.POINTER(_dbl)]),
    ("ozgb_choose_slices_ex", _i, [_p, _p, _i, _p, _p, _i, _p, _p, _i, _i, _dbl, _i, _dbl, ctypes.POINTER(_dbl)]),
    ("ozgb_dgemm_device_noalloc", _i, [_i, _i, _i, _p, ctypes.c_long, _p, ctypes.c_long, _p, ctypes.c_long, _i, _p]),
    ("ozgb_dgemm_ex", _i, [_h, _i, _i, _i, _i, _i, _dbl, _p, ctypes.c_long, _p, ctypes.c_long, _dbl, _p,
                           ctypes.c_long, _p]),
    ("ozgb_dump_pairs", _i, [_h, _i, _i, _i, _p, _p, _p]),
    ("ozgb_autotune", _i, [_h, _i, _i, _i, _i, _i, _i, _i, ctypes.POINTER(OzgbConfig)]),
    ("ozgb_tuning_entries", _i, []),
    ("ozgb_tuning_clear", None, []),
    ("ozgb_launch_count", _i, [_h, ctypes.POINTER(ctypes.c_longlong)]),
    ("ozgb_version", ctypes.c_char_p, []),
]


def lib_path():
    """liboz_gb300.so in the package directory, or the path in OZGB_LIB_PATH
    (an alternative build of the same library)."""
    return os.environ.get("OZGB_LIB_PATH") or _build.LIB


def load(build_if_missing=True):
    """Load liboz_gb300.so (building it first if absent and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError("liboz_gb300.so is not built; run ozaie_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return _lib


class OzgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code
