/*
 * oz_gb300.h -- C ABI of the GB300 Ozaki-scheme DGEMM library (liboz_gb300.so).
 *
 * Plain C types only (ints, doubles, pointers, an opaque handle).  The drop-in
 * C++ header include/oz_aie.h is written on top of these functions, and the
 * Python package ozaie_gb300 binds them with ctypes.
 *
 * Reference interface replaced (atlarge-research/ozAIE):
 *   oz_aie::ozAIE_setup            include/oz_aie.h:182-300  -> ozgb_setup
 *   oz_aie::ozAIE_DGEMM            include/oz_aie.h:311-349  -> ozgb_dgemm
 *   oz_aie::convert_paired_i64_to_double_matrix
 *                                  include/oz_aie.h:92-150   -> ozgb_convert_paired_i64_to_double
 *   oz_aie::cleanup_xrt            include/oz_aie.h:153-170  -> ozgb_release
 *   process-global state b, d, buffers (include/oz_aie.h:31-58) -> ozgb_handle
 *
 * Every function returns an ozgb_status (0 = success).  No function falls back
 * to the CPU: without a usable CUDA device the compute entry points return
 * OZGB_ERR_NO_DEVICE.
 *
 * Handles: calls on one handle are serialised on the host (a mutex) and reuse
 * the handle's device buffers (exponents, slice planes, split sums), so two
 * calls on one handle must not overlap on the GPU: give each stream its own
 * handle.  Buffers grow on first use (cudaMalloc); warm a handle up before
 * capturing its calls in a CUDA graph.
 */
#ifndef OZ_GB300_H
#define OZ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ozgb_context *ozgb_handle;

typedef enum {
    OZGB_OK = 0,
    OZGB_ERR_DIMS = 1,          /* bad dimensions; ozAIE_setup's status 1 (include/oz_aie.h:187-191) */
    OZGB_ERR_NO_DEVICE = 2,     /* no usable CUDA device; takes the place of ozAIE_setup's 2 (missing env) */
    OZGB_ERR_EXEC = 3,          /* a kernel failed to launch or run; ozAIE_DGEMM's 3 (include/oz_aie.h:337-340) */
    OZGB_ERR_IMAGE = 4,         /* no kernel image for this GPU; takes the place of ozAIE_setup's 4 (build failed) */
    OZGB_ERR_NOT_SETUP = 5,     /* ozgb_dgemm called before ozgb_setup */
    OZGB_ERR_DIM_MISMATCH = 6,  /* ozgb_dgemm dims differ from the last setup (the reference overruns its buffers) */
    OZGB_ERR_ARG = 7,           /* null pointer or invalid option value */
    OZGB_ERR_ALLOC = 8,         /* device memory allocation failed */
    OZGB_ERR_TIMEOUT = 9,       /* a device-side wait ran out of time; the kernel stopped early */
    OZGB_ERR_UNSUPPORTED = 10,  /* the requested slices/bins exceed the exact-accumulation limits */
    OZGB_ERR_TOO_LARGE = 11     /* ozgb_dgemm_device_noalloc: the problem needs more than its fixed scratch */
} ozgb_status;

typedef enum { OZGB_MODE_ACCURATE = 0, OZGB_MODE_FAST = 1 } ozgb_mode; /* oz_aie::Mode, include/oz_aie.h:82 */

typedef enum {
    OZGB_PROFILE_GB300 = 0,     /* fast: b=7, s=8, triangular; accurate: b=7, s=8, full pair set; RN */
    OZGB_PROFILE_REFERENCE = 1  /* the reference's (b, d) tables (include/oz_aie.h:60-80), triangular, RZ decode */
} ozgb_profile;

typedef enum {
    OZGB_ROUND_DEFAULT = -1,     /* profile's choice */
    OZGB_ROUND_NEAREST = 0,      /* exact bin sum rounded to nearest even, IEEE subnormals/overflow */
    OZGB_ROUND_REFERENCE = 1     /* the reference's truncating decode (include/oz_aie.h:124-146) */
} ozgb_rounding;

/* Effective configuration of the last setup / call. */
typedef struct {
    int bits;        /* b: magnitude bits per slice */
    int slices;      /* s (the reference's d / num_splits) */
    int bins;        /* J: pair set {p + q <= J - 1}; J = s triangular, J = 2s - 1 full */
    int rounding;    /* ozgb_rounding */
    int tile_n;      /* BN of the slice-pair GEMM */
    int k_chunk;     /* K elements per pipeline stage */
    int stages;      /* pipeline stages */
    int drain_chunks;/* K chunks accumulated in fp32 before a drain (exactness period) */
    int acc_words;   /* 32-bit words of the exact per-element accumulator */
    int pairs;       /* slice-pair products per K step */
    int blocks;      /* bin blocks (one UMMA accumulator range each) */
    int umma_per_kstep; /* UMMAs per 16-deep K step */
    int block_lo[8]; /* first bin of each block */
    int block_nb[8]; /* bins in each block */
    int issuers;     /* warps issuing the UMMAs (1 to 3; the UMMA runs of a K step dealt round-robin) */
    int slice_format;/* 0: bf16 slices (kind::f16); 1: e4m3 slices (kind::f8f6f4, b <= 4) */
    int dbl_blocks;  /* bit g: block g has two accumulator ranges, its UMMAs go on while one drains */
} ozgb_config;

/* ---------------------------------------------------------------- handles */
ozgb_status ozgb_create(ozgb_handle *out);
ozgb_status ozgb_destroy(ozgb_handle h);
/* Frees device buffers, keeps options; counterpart of cleanup_xrt (include/oz_aie.h:153-170). */
ozgb_status ozgb_release(ozgb_handle h);

/* ------------------------------------------------------------ drop-in path */
/* ozAIE_setup (include/oz_aie.h:182): picks (b, s, J) for `mode` and sizes device
 * buffers.  Accepts any M, N, K >= 1 (a superset of the reference's square
 * power-of-two 128..2048). */
ozgb_status ozgb_setup(ozgb_handle h, int M, int N, int K, int mode);
/* ozAIE_DGEMM (include/oz_aie.h:311): C = A B on row-major host arrays
 * (alpha = 1, beta = 0, C overwritten).  Dims must equal the last setup. */
ozgb_status ozgb_dgemm(ozgb_handle h, int M, int N, int K, const double *A, const double *B, double *C);

/* --------------------------------------------------------- device pointers */
/* Same product on device arrays with leading dimensions, enqueued on `stream`
 * (a cudaStream_t; NULL = the CUDA default stream).  Returns after enqueueing;
 * ozgb_sync() reports device-side errors.  Uses the mode of the last setup
 * (or OZGB_MODE_FAST when there was none). */
ozgb_status ozgb_dgemm_device(ozgb_handle h, int M, int N, int K, const double *dA, long lda,
                              const double *dB, long ldb, double *dC, long ldc, void *stream);
/* BLAS-style form on device arrays, row-major like the rest of the API:
 *   C = alpha * op(A) op(B) + beta * C,  op(A) M x K, op(B) K x N,
 * op(A) = A (stored M x K, lda >= K) or, with transa, A^T (A stored K x M,
 * lda >= M); op(B) likewise (transb: B stored N x K, ldb >= K).  The product is
 * the exact Ozaki result rounded once; alpha and beta are then applied in FP64
 * (C is not read when beta == 0; A and B are not read when alpha == 0).  No
 * reference counterpart: the reference computes C = A B on host arrays only
 * (include/oz_aie.h:311). */
ozgb_status ozgb_dgemm_ex(ozgb_handle h, int transa, int transb, int M, int N, int K, double alpha, const double *dA,
                          long lda, const double *dB, long ldb, double beta, double *dC, long ldc, void *stream);
/* Waits for the last enqueued call and checks the device error word. */
ozgb_status ozgb_sync(ozgb_handle h);

/* ------------------------------------------------- no device allocation */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * code inside another framework's memory pool or caching allocator, code that
 * must not trigger the device synchronisation of cudaMalloc/cudaFree, code with
 * a memory budget fixed in advance.  Same product as ozgb_dgemm_device (device
 * arrays, leading dimensions, enqueued on `stream`, NULL = default stream) with
 * b = 7, `slices` in [2, 16], triangular pair set, round to nearest; no handle.
 * All scratch comes from one 64 MiB static device array reserved when the
 * library loads; a product needs about 4 (M + N) + 2 s (Mp + Np) Kp bytes
 * (Mp, Np, Kp: M, N, K rounded up to the tile sizes), e.g. 1024^3 up to s = 15,
 * 2048 x 2048 x 1024 up to s = 7.  Larger products return OZGB_ERR_TOO_LARGE.
 * The first call on a device (with it current) sets up the array's address:
 * make that first call before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race.  Device-side wait timeouts (a stalled
 * GPU) leave C incomplete and are not reported here; ozgb_dgemm_device with
 * ozgb_sync reports them. */
ozgb_status ozgb_dgemm_device_noalloc(int M, int N, int K, const double *dA, long lda, const double *dB, long ldb,
                                      double *dC, long ldc, int slices, void *stream);

/* --------------------------------------------------------------- grouped */
typedef struct {
    int M, N, K;
    const double *A; long lda; /* device pointers */
    const double *B; long ldb;
    double *C; long ldc;
    double error_bound; /* requested normwise relative error; <= 0: use the handle's slices */
    int slices_used;    /* out: slices chosen for this problem */
    int bins_used;      /* out: its pair set, p + q <= bins_used - 1 */
} ozgb_problem;
/* Many independent DGEMMs of any sizes (the spec batched form; the
 * reference runs one ozAIE_DGEMM per call, include/oz_aie.h:311).  One launch
 * computes the exponents of every problem, one the splits of every problem; the
 * slice-pair GEMMs run per problem, largest first, on auxiliary streams forked
 * from and joined back into `stream`.  Problems with an error bound get their
 * slice count from the precision knob: the call then waits once for the knob's
 * statistics of all problems.  With ozgb_set_graph(h, 1) both halves are
 * captured into CUDA graphs and replayed while the problem list (sizes,
 * pointers, bounds) and the chosen slice counts stay the same.  The handle's
 * grouped buffers serve one call at a time: calls on one handle must not
 * overlap on the GPU. */
ozgb_status ozgb_dgemm_grouped(ozgb_handle h, ozgb_problem *probs, int n, void *stream);

/* ---------------------------------------------------------------- options */
ozgb_status ozgb_set_profile(ozgb_handle h, int profile);
ozgb_status ozgb_set_bits(ozgb_handle h, int bits);        /* 0 = profile default */
ozgb_status ozgb_set_slices(ozgb_handle h, int slices);    /* 0 = profile default */
ozgb_status ozgb_set_bins(ozgb_handle h, int bins);        /* 0 = default, -1 = full pair set, else J */
ozgb_status ozgb_set_rounding(ozgb_handle h, int rounding);
/* Slice format: 0 = e4m3 where it is exact (b <= 4) and a kernel fits, else bf16
 * (default); 1 = bf16 always. */
ozgb_status ozgb_set_slice_format(ozgb_handle h, int format);
/* Fixes choices of the slice-pair GEMM plan for this handle's single calls (0 =
 * the planner's choice): tile width tile_n (16..128), K chunk, pipeline stages,
 * issuing warps (1 to 3), double-buffered blocks (dbl: -1 the planner's
 * choice, 0 none, 1 every block that fits TMEM), and `blocks` bin-block sizes
 * block_nb[0..blocks) covering the bins.  All zeros and dbl = -1 clear it.  A
 * call whose plan cannot honour the hint fails with OZGB_ERR_UNSUPPORTED. */
ozgb_status ozgb_set_plan_hint(ozgb_handle h, int tile_n, int k_chunk, int stages, int issuers, int dbl, int blocks,
                               const int *block_nb);
/* Requested relative error (> 0 enables slice selection from the exponent
 * spread measured by stage (a)); 0 disables it.  The error it bounds is set by
 * ozgb_set_error_criterion (normwise by default). */
ozgb_status ozgb_set_error_bound(ozgb_handle h, double bound);
/* Which error the precision knob bounds.  No reference counterpart (the
 * reference fixes s per shape, include/oz_aie.h:60-80; its harness reports the
 * largest elementwise relative error against MPFR, common.h:585-592).
 *   OZGB_CRIT_NORMWISE (default): |C^ - C|_F / |C|_F.
 *   OZGB_CRIT_ELEMENTWISE: |c^_ij - c_ij| / |c_ij| for every entry with
 *     |c_ij| >= tail * |a_i| |b_j| / sqrt(K) (row i of op(A), column j of
 *     op(B)).  An entry that cancels to near zero has no relative error bound at
 *     any fixed precision; `tail` (in (0, 1], e.g. 1e-4) leaves out the entries
 *     within that distance of zero, about a tail's fraction of them for random
 *     signs and moderate spreads. 
 * Both are a-priori estimates from the stage-(a) statistics, not guarantees. */
enum { OZGB_CRIT_NORMWISE = 0, OZGB_CRIT_ELEMENTWISE = 1 };
ozgb_status ozgb_set_error_criterion(ozgb_handle h, int criterion, double tail);
/* The slice schedule the precision knob searches.  1 (default): every slice
 * count s in [2, 16] and pair set p + q <= J - 1 with s <= J <= 2s - 1; the
 * knob takes the schedule with the smallest modelled time (the GEMM's UMMA
 * count on this device plus the split's traffic) whose estimate meets the bound.
 * 0: the triangular set J = s only (the reference's pair set,
 * src/aie_kernels/aie2p/mm_ozaki.cc:255-308), smallest s. */
ozgb_status ozgb_set_schedule_search(ozgb_handle h, int any_pair_set);
ozgb_status ozgb_set_graph(ozgb_handle h, int enable);     /* capture grouped calls in CUDA graphs */
/* Grouped calls' slice-pair GEMMs: 1 (default) = one persistent launch per plan
 * class (the problems whose plans share the kernel variant, stage layout, bin
 * blocks, drain schedule and accumulator groups), its CTAs walking the tiles of
 * all of its problems, largest problems first; 0 = one launch per problem. */
ozgb_status ozgb_set_grouped_launch(ozgb_handle h, int mode);
ozgb_status ozgb_set_timeout_ms(ozgb_handle h, double ms); /* device-side wait limit, default 2000 */
ozgb_status ozgb_get_config(ozgb_handle h, ozgb_config *out);
/* Per-stage device times of the last call (ms): [0] exponents, [1] split,
 * [2] slice-pair GEMM + accumulation, [3] total.  Needs ozgb_set_profiling(h, 1). */
ozgb_status ozgb_set_profiling(ozgb_handle h, int enable);
ozgb_status ozgb_stage_times(ozgb_handle h, float *ms, int n);
/* Number of kernels this handle has launched so far (all entry points).  No
 * reference counterpart: lets a caller check that its calls ran on the GPU. */
ozgb_status ozgb_launch_count(ozgb_handle h, long long *count);
const char *ozgb_last_error(ozgb_handle h);

/* -------------------------------------------------------- test / debug hooks */
/* Intermediates of one DGEMM on host arrays, for parity checks:
 *  er[M], ec[N]            max exponents (stage a), may be NULL
 *  a_slices[s][M][K]       int8 slices of A (stage b), may be NULL
 *  b_slices[s][K][N]       int8 slices of B, may be NULL
 *  q[M][N][4]              exact per-element accumulator as 128-bit two's
 *                          complement (4 little-endian 32-bit words), for bins
 *                          [bin_lo, bin_hi] only (stage c); may be NULL
 * Uses the handle's current options (setup dims need not match). */
ozgb_status ozgb_dump(ozgb_handle h, int M, int N, int K, const double *A, const double *B, int32_t *er,
                      int32_t *ec, int8_t *a_slices, int8_t *b_slices, int32_t *q, int bin_lo, int bin_hi);
/* Runs a kernel whose only wait is on an mbarrier that nothing arrives on, with
 * the given limit; returns OZGB_ERR_TIMEOUT when the bounded wait gave up and the
 * device stayed usable (tests the timeout path without faulting the GPU). */
ozgb_status ozgb_selftest_timeout(ozgb_handle h, double timeout_ms);
/* The reference's device output for A B (host arrays, the handle's profile and
 * mode; triangular pair set): pairs[(row * N + col) * 2] = lo and [+1] = hi, the
 * two int64 sums of ozaki_vectorized_sum_upshift (ozaki_base.cc:143-340) with
 * Er + Ec in bits 51..62 of hi -- the buffer that ozAIE_DGEMM reads back before
 * convert_paired_i64_to_double_matrix (include/oz_aie.h:342-346). */
ozgb_status ozgb_dump_pairs(ozgb_handle h, int M, int N, int K, const double *A, const double *B, int64_t *pairs);

/* Host helper kept from the reference: decodes the 2 x int64 per element wire
 * format (include/oz_aie.h:92-150), C[row*(2N) + 2col] = low, +1 = high. */
ozgb_status ozgb_convert_paired_i64_to_double(const int64_t *C, double *result, int M, int N, int K,
                                              int num_splits, int bits_per_slice);

/* Autotuner (no reference counterpart; the reference fixes its tiling per
 * shape).  Times up to max_candidates feasible plans (tile width, K chunk,
 * number of bin blocks, pipeline depth) of the slice-pair GEMM for an M x N x K
 * product with `bits`, `slices`, `bins` (0 = slices, the triangular set) on
 * this handle's device, with pseudo-random operands, and records the fastest in
 * a process-wide table keyed by (bits, slices, bins, rounding, ceil(log2) of
 * M, N, K).  Later calls of any handle with a matching configuration use it.
 * Writes the winner to *best (may be NULL).  Allocates device memory. */
ozgb_status ozgb_autotune(ozgb_handle h, int M, int N, int K, int bits, int slices, int bins, int max_candidates,
                          ozgb_config *best);
/* Number of entries in the tuning table; clearing it restores the planner's
 * cost-model choices. */
int ozgb_tuning_entries(void);
void ozgb_tuning_clear(void);

/* Host-only planning query (no device needed): the kernel configuration the
 * library would use for an M x N x K product with `bits`, `slices`, `bins`. */
int ozgb_plan_query(int M, int N, int K, int bits, int slices, int bins, ozgb_config *out);
/* Host-only precision knob (no device needed): the smallest slice count in
 * [2, 16] whose a-priori normwise error estimate is <= bound (16 if none), from
 * the stage-(a) statistics: row max exponent fields er and row sums of squares
 * ssr of A, column fields ec and column sums of squares ssc of B, and the sums
 * of squares along k, sa_k[k] = |A(:,k)|^2 and sb_k[k] = |B(k,:)|^2 (both may be
 * NULL: the mass of A and B is then taken as spread evenly over k).  The
 * device path computes the same statistics itself.  No reference counterpart:
 * the reference fixes s per shape (include/oz_aie.h:60-80).  Returns -1 on bad
 * input. */
int ozgb_choose_slices(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                       const double *sa_k, const double *sb_k, int K, int bits, double bound, double *estimate);
/* Host-only slice schedule (no device needed): the (slices, bins) the knob picks
 * on a device with `sms` SMs for an M x N x K product with these statistics,
 * criterion and tail (ozgb_set_error_criterion) and search (ozgb_set_schedule_search).
 * Returns 0, or -1 on bad input. */
int ozgb_choose_schedule(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                         const double *sa_k, const double *sb_k, int K, int bits, double bound, int criterion,
                         double tail, int any_pair_set, int sms, int *slices, int *bins, double *estimate);
/* The same with a criterion and tail as in ozgb_set_error_criterion. */
int ozgb_choose_slices_ex(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                          const double *sa_k, const double *sb_k, int K, int bits, double bound, int criterion,
                          double tail, double *estimate);

/* Host-only check of the grouped launches (no device needed, a test hook): the
 * launches that ozgb_dgemm_grouped would make for these problems (b = 7,
 * `slices`, `bins`, round to nearest; A, B unused; C pointers and ldc as given)
 * are built with stand-in device addresses, and every work unit is walked as the
 * kernel walks it: each tile of each problem exactly once, every bulk copy inside
 * the problem's slice blocks, the epilogue's C and exponents those of its
 * problem.  Returns 0 and the number of launches and work units, or a negative
 * code naming the first violated check. */
int ozgb_grouped_layout_check(const ozgb_problem *probs, int n, int slices, int bins, int *launches_out,
                              long long *units_out);

/* Library version string. */
const char *ozgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OZ_GB300_H */
