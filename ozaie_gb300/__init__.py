"""oz-gb300: Ozaki-scheme DGEMM emulation on one NVIDIA GB300 (sm_103a).

The compute path is liboz_gb300.so (hand-written CUDA, C ABI in
include/oz_gb300.h); this package binds it with ctypes and mirrors the
reference's ozAIE_setup / ozAIE_DGEMM API.
"""
from .api import (Criterion, Handle, Mode, Profile, Rounding, choose_schedule, choose_slices, cleanup_xrt, convert_paired_i64_to_double_matrix,
                  grouped_layout_check, ozAIE_DGEMM, ozAIE_setup, plan_query, q_words_to_int)
from ._lib import OzgbError, load

__all__ = [
    "Criterion", "Handle", "Mode", "Profile", "Rounding", "OzgbError", "load", "ozAIE_setup", "ozAIE_DGEMM", "cleanup_xrt",
    "convert_paired_i64_to_double_matrix", "plan_query", "choose_schedule", "choose_slices", "q_words_to_int",
    "grouped_layout_check",
]
