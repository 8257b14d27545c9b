/*
 * oz_oracle.h -- CPU restatement of the Oz-AIE Ozaki-scheme arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py load it.  The
 * product path (ozaie_gb300/liboz_gb300.so) never links or calls it.
 *
 * Parity status of each stage against the reference (atlarge-research/ozAIE):
 *   (d-host) decode of the 2 x int64 wire format: PINNED.  tests/ compare
 *            ozo_decode_pairs() bit-for-bit with the reference's own
 *            convert_paired_i64_to_double_matrix (include/oz_aie.h:92-150),
 *            compiled from the reference sources into oracle/_ref/.
 *   (a) exponent max, (b) split, (c) slice-pair bins, (d-device) bin sum:
 *            PARITY UNPINNED.  The reference ships no golden vectors for them
 *            and its AIE kernels need the aie_api / Peano toolchain, which is
 *            not available, so they cannot be executed here.  They are
 *            restated line by line from ozaki_base.cc and aie2p/mm_ozaki.cc.
 *
 * Layouts: all matrices are row-major; slice planes are [d][rows][cols] int8.
 */
#ifndef OZ_ORACLE_H
#define OZ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Stage (a): running max of the 11-bit biased exponent field, start value 0.
 * ozaki_base.cc:342-440 (rows of A); same kernel applied to columns of B. */
void ozo_max_exp_rows(const double *A, int M, int K, int32_t *Er);
void ozo_max_exp_cols(const double *B, int K, int N, int32_t *Ec);

/* Stage (b): split one double into d signed slices of b bits, aligned to the
 * max exponent E.  ozaki_base.cc:449-639 (extract_splits_acc64_half_half). */
void ozo_split_elem(uint64_t x_bits, int E, int b, int d, int8_t *out, long stride);
/* Split every row of A [M][K] into planes [d][M][K]. */
void ozo_split_rows(const double *A, int M, int K, const int32_t *Er, int b, int d, int8_t *planes);
/* Split every column of B [K][N] into planes [d][K][N]. */
void ozo_split_cols(const double *B, int K, int N, const int32_t *Ec, int b, int d, int8_t *planes);

/* Stage (c): bins[j][m][n] = sum_{p+q=j, p<d, q<d, j<J} sum_k A_p[m,k] B_q[k,n], exact
 * in int64.  J = d is the reference's triangular set (aie2p/mm_ozaki.cc:283-305);
 * J = 2d-1 is the full set.  OpenMP over rows. */
void ozo_bins(const int8_t *Ap, const int8_t *Bp, int M, int N, int K, int d, int J, int64_t *bins);

/* Stage (d, device side): the reference's 2 x int64 per C element
 * (ozaki_base.cc:143-340): lo/hi group sums of the int32 bins plus the exponent
 * scale-back embedded in bits 51..62 of hi.  bins are taken modulo 2^32 as the
 * reference's int32 bins.  Output pairs[m][n][2] = {lo, hi}. */
void ozo_sum_upshift(const int64_t *bins, const int32_t *Er, const int32_t *Ec, int M, int N, int K,
                     int b, int d, int64_t *pairs);
/* First-group size g0 of the 2 x int64 format (ozaki_base.cc:151-158). */
int ozo_first_group(int K, int b, int d);

/* Stage (d, host side): restatement of convert_paired_i64_to_double_matrix
 * (include/oz_aie.h:92-150): int128 = lo + sext51(hi) << (g0 b), truncated (RZ). */
void ozo_decode_pairs(const int64_t *pairs, double *C, int M, int N, int K, int d, int b);

/* GB300 finishing rule: q = sum_j bins_j 2^{b(J-1-j)} exactly (no 2 x int64
 * wire format), value = q 2^{Er+Ec-2044-b(J+1)}.
 * rounding 0: round to nearest even with IEEE subnormals / infinities.
 * rounding 1: the reference's truncating decode arithmetic applied to q.
 * q_out (optional, may be NULL): q as 4 little-endian int64 words (two's complement). */
void ozo_finish(const int64_t *bins, const int32_t *Er, const int32_t *Ec, int M, int N, int b, int J,
                int rounding, double *C, int64_t *q_out);

/* Whole pipeline (a)->(d) for one DGEMM, C = A B. */
void ozo_dgemm(const double *A, const double *B, double *C, int M, int N, int K, int b, int d, int J,
               int rounding);
/* Pipeline restricted to rows [r0, r1) of A (CPU-baseline samples). Exponents
 * still cover all of K; column exponents of B are computed over all of B. */
void ozo_dgemm_rows(const double *A, const double *B, double *C, int M, int N, int K, int b, int d,
                    int J, int rounding, int r0, int r1);

/* Exact reference: for each (rows[i], cols[i]) the exact sum_k A B rounded to
 * nearest double (Kulisch-style fixed-point accumulator), and sum_k |A||B|. */
void ozo_exact_entries(const double *A, const double *B, int M, int N, int K, const int32_t *rows,
                       const int32_t *cols, int n, double *out, double *absdot);

/* MPFR oracle at prec bits, mirroring mul_acc_MPFR (common.h:211-232): running
 * sum rounded to prec bits after every multiply and add.  libmpfr.so.6 is loaded
 * with dlopen; returns -1 when it is not available, 0 otherwise. */
int ozo_mpfr_entries(const double *A, const double *B, int M, int N, int K, const int32_t *rows,
                     const int32_t *cols, int n, int prec, double *out);

/* Naive triple-loop DGEMM (common.h:234-254), single thread. */
void ozo_dgemm_naive(const double *A, const double *B, double *C, int M, int N, int K);

/* Threads used by the OpenMP loops (0 when built without OpenMP). */
int ozo_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
