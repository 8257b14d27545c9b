// oz_aie.h -- drop-in replacement for the Oz-AIE public C++ API, backed by the
// GB300 library (liboz_gb300.so, C ABI in oz_gb300.h).
//
// Same namespace, enum, function names, argument meaning and status codes as the
// reference header (atlarge-research/ozAIE include/oz_aie.h):
//   enum Mode { accurate = 0, fast = 1 }                         (:82)
//   int32_t ozAIE_setup(int M, int N, int K, enum Mode mode)     (:182-300)
//   int32_t ozAIE_DGEMM(int M, int N, int K, const double *A,
//                       const double *B, double *C)              (:311-349)
//   void convert_paired_i64_to_double_matrix(...)                (:92-150)
//   void cleanup_xrt()                                           (:153-170)
// Differences, all supersets of the reference behaviour:
//   * any M, N, K >= 1 (the reference accepts only square powers of two in
//     [128, 2048]; status 1 for anything else);
//   * status 2 means "no usable CUDA device" (the reference: missing environment);
//   * ozAIE_DGEMM returns 6 when the dimensions differ from the last setup (the
//     reference silently overruns its buffers), 5 when setup was never called;
//   * every function is inline: the header can be included by several
//     translation units (the reference defines non-inline globals).
// Link with liboz_gb300.so (include/CMakeLists.txt provides use_ozaie(target)).
#pragma once

#include <cstdint>

#include "oz_gb300.h"

namespace oz_aie {

enum Mode { accurate = 0, fast = 1 };

namespace detail {
// The reference keeps process-global state (include/oz_aie.h:31-58); one
// library handle plays that role here.
inline ozgb_handle &handle() {
    static ozgb_handle h = nullptr;
    if (!h) ozgb_create(&h);
    return h;
}
}  // namespace detail

/// Converts the 2 x int64 per element wire format to doubles (reference
/// include/oz_aie.h:92-150): C[row*(2N) + 2col] = low, +1 = high.
inline void convert_paired_i64_to_double_matrix(int64_t *C, double *result, int M, int N, int K, int num_splits,
                                                int bits_per_slice) {
    ozgb_convert_paired_i64_to_double(C, result, M, N, K, num_splits, bits_per_slice);
}

/// Releases the device buffers of the previous setup (reference cleanup_xrt).
inline void cleanup_xrt() {
    if (detail::handle()) ozgb_release(detail::handle());
}

/// Prepares an M x N x K Ozaki-scheme DGEMM in the given mode.  Returns 0 on
/// success, 1 for non-positive dimensions, 2 without a usable CUDA device.
inline int32_t ozAIE_setup(int M, int N, int K, enum Mode mode) {
    ozgb_handle h = detail::handle();
    if (!h) return OZGB_ERR_ALLOC;
    return static_cast<int32_t>(ozgb_setup(h, M, N, K, static_cast<int>(mode)));
}

/// C = A B for row-major host arrays (alpha = 1, beta = 0).  Returns 0 on
/// success, 3 when execution failed on the device.
inline int32_t ozAIE_DGEMM(int M, int N, int K, const double *A, const double *B, double *C) {
    ozgb_handle h = detail::handle();
    if (!h) return OZGB_ERR_ALLOC;
    return static_cast<int32_t>(ozgb_dgemm(h, M, N, K, A, B, C));
}

}  // namespace oz_aie
