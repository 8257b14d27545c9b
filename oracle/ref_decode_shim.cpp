// ref_decode_shim.cpp -- C entry point around the reference's own host decode.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_oracle.py extracts the body of
// convert_paired_i64_to_double_matrix from the reference's include/oz_aie.h
// (lines 92-150 at the pinned revision) into oracle/_ref/ref_decode_body.inc at
// build time; this file compiles that text unchanged inside its own namespace so
// the oracle's restatement (ozo_decode_pairs) can be checked against it.  The
// rest of oz_aie.h needs XRT and cannot be compiled here.
#include <sys/types.h>

#include <algorithm>
#include <bit>
#include <cstdint>
#include <iostream>

namespace ozref {
#include "_ref/ref_decode_body.inc"
}

extern "C" void ref_convert_paired_i64_to_double_matrix(int64_t *C, double *result, int M, int N, int K,
                                                        int num_splits, int bits_per_slice) {
    ozref::convert_paired_i64_to_double_matrix(C, result, M, N, K, num_splits, bits_per_slice);
}
