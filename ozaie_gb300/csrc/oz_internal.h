// oz_internal.h -- shared definitions of the GB300 Ozaki DGEMM kernels and host code.
//
// Data layout in HBM (written by stage (b), read by stage (c)):
//   A slices: for each 128-row tile mt and K chunk c, the s slices of that block
//     are one contiguous region  [mt][c][p][128 rows x KC]  of bf16, and
//   B slices (of B^T, i.e. N rows with K contiguous):  [nt][c][q][BN rows x KC].
//   Inside a (rows x KC) block the elements follow the tcgen05 K-major canonical
//   layout without swizzle: 8-row x 8-element (16-byte) core matrices, the core
//   matrices of an 8-row group consecutive along K (LBO = 128 B), 8-row groups
//   KC*16 bytes apart (SBO).  One bulk copy moves a whole stage.
#pragma once
#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define OZ_HD __host__ __device__
#else
#define OZ_HD
#endif

namespace ozgb {

constexpr int BM = 128;         // rows of A per tile (UMMA M)
constexpr int kMaxBins = 64;      // J limit
constexpr int kMaxGroups = 8;     // drain groups limit
constexpr int kMaxAcc = 4;        // 64-bit accumulator groups per element (drain)
constexpr int kEpiWarps = 16;     // drain + epilogue warps: 4 per TMEM lane quadrant
// warp 0 producer, warp 1 MMA issuer, then the drain warps, then two more MMA
// issuers, so that the issuing warps sit on three different schedulers: one thread
// issues a UMMA about every 80-100 SM cycles, while the tensor pipe takes N / 2
// cycles for one of N columns, so narrow UMMAs need several issuers to keep it
// busy.  (640 threads keep ptxas's register limit at 96 per thread.)
constexpr int kThreads = 64 + 32 * kEpiWarps + 64;
constexpr int kIssuer2Warp = 2 + kEpiWarps;  // issuing warps: 1, kIssuer2Warp and kIssuer2Warp + 1
constexpr int kMaxIssuers = 3;
constexpr int kMaxAccWords = 5;

// OUT_PAIRS writes the reference's device output (its C buffer before the host
// decode): per element int64 lo, hi with (Er + Ec) in bits 51..62 of hi.
enum OutMode : int { OUT_RN = 0, OUT_RZ_REF = 1, OUT_RAW = 2, OUT_PAIRS = 3 };

// Shared memory after the pipeline stages: mbarriers, TMEM slot, abort flag
// (plus 1 KB of alignment slack).
constexpr size_t kCtrlBytes = 1024 + 1024;

// Element offset of (row r, k) inside one (rows x KC) canonical block.
OZ_HD inline long canon_offset(int r, int kk, int KC) {
    return (long)(((r >> 3) * (KC >> 3) + (kk >> 3)) * 64 + (r & 7) * 8 + (kk & 7));
}
// The same layout for one-byte (e4m3) slices: 16 K values per core-matrix row, so a
// 64-deep e4m3 chunk has the byte layout of a 32-deep bf16 chunk.
OZ_HD inline long canon_offset8(int r, int kk, int KC) {
    return (long)(((r >> 3) * (KC >> 4) + (kk >> 4)) * 128 + (r & 7) * 16 + (kk & 15));
}

// One problem of a grouped slice-pair GEMM launch (GemmArgs::probs): every
// problem of the launch shares the kernel variant, the stage layout, the bin
// blocks, the drain schedule and the accumulator groups; these are its own.
struct GroupProblem {
    const uint8_t *a_tiles;  // its A slice blocks: [tiles_m][n_kc] blocks of a_block_bytes
    const uint8_t *b_tiles;  // its B slice blocks: [tiles_n][n_kc] blocks of b_block_bytes
    const int32_t *er;
    const int32_t *ec;
    double *c;
    long ldc;
    int M, N, n_kc, tiles_m, tiles_n;
    int tile0;  // its first work unit in the launch
};

struct GemmArgs {
    const uint16_t *a_tiles;
    const uint16_t *b_tiles;
    const int32_t *er;
    const int32_t *ec;
    double *c;
    long ldc;
    int32_t *raw;  // OUT_RAW: [M][N][4] words; OUT_PAIRS: [M][N][2] int64
    int M, N;
    int n_kc, KC, s, J, b;
    int out_mode;
    int tiles_m, tiles_n;
    int stages;
    // Stage layout: [A: s slices of BM x KC][B region: pad_lo zero slices, the s
    // loaded B slices, pad_hi zero slices], each B slice BN x KC.
    uint32_t stage_bytes, a_block_bytes, b_block_bytes, b_pad_lo_bytes, b_region_bytes;
    uint32_t tmem_cols;
    int *err;
    unsigned long long timeout_ns;
    // Bin blocks (also the drain groups).  Block g holds bins [lo, lo + nb);
    // every UMMA of the block covers all of its bins (one accumulator range):
    // A slice p in [p0, p1] against B slices q = j - p, the out-of-range q
    // reading zero slices.  Block g is drained after chunk c when
    // (c + 1 + off) % period == 0, and after the last chunk.
    int G;
    int blk_lo[kMaxGroups], blk_nb[kMaxGroups], blk_p0[kMaxGroups], blk_p1[kMaxGroups];
    int blk_period[kMaxGroups], blk_off[kMaxGroups];
    // Double-buffered blocks (bit g of dbl_mask): a second accumulator range at
    // TMEM column blk_col1[g]; after each drain the block's UMMAs switch ranges,
    // so they go on while the drain warps read the other one out.
    uint32_t dbl_mask;
    int blk_col1[kMaxGroups];
    int total_tiles;  // end of the launch's tile range (tiles_m * tiles_n for the whole product)
    int tile_begin;   // first tile of the launch's range (0 for the whole product)
    // Grouped launch (null otherwise): work unit u < total_tiles is tile
    // u - probs[p].tile0 of problem p = tile_prob[u]; the per-problem fields above
    // (operands, sizes, tiles) are then unused.  No K-split in grouped launches.
    const GroupProblem *probs;
    const int *tile_prob;
    // Split of the launch's last partial wave along K: work unit u < split_start is
    // tile u over all of K; unit u >= split_start is part (u - split_start) %
    // split_parts of tile split_start + (u - split_start) / split_parts, over chunks
    // [part n_kc / P, (part + 1) n_kc / P).  Each part adds its 64-bit group sums
    // into split_acc (per split tile: [NA][BN][128], zero before the launch) and
    // counts itself in split_cnt; the part that completes the count rounds and
    // stores the tile.  total_tiles is then the end of the unit range.
    int split_start, split_parts;
    unsigned long long *split_acc;
    int *split_cnt;
    int pair_g0;      // OUT_PAIRS: bins in the low word group (the reference's first group)
    // Accumulator groups of the drain: with t = J - 1 - j, bin j is added into the
    // 64-bit accumulator a of its group (the last a with acc_t0[a] <= t) with
    // weight 2^(b (t - acc_t0[a])); the exact sum is sum_a acc_a 2^(b acc_t0[a]).
    // The planner keeps every weight <= 2^30 and every group's worst-case sum
    // below 2^63.  OUT_PAIRS: groups {0, pair_g0}, each modulo 2^64.
    int n_acc;
    int acc_t0[kMaxAcc];
    int n_iss;  // MMA-issuing warps (1 to 3): the UMMA runs of a K step are dealt round-robin
    double alpha, beta;  // C = alpha * (A B) + beta * C for OUT_RN / OUT_RZ_REF (1, 0: plain store)
};

// Partial sums of squares of reduction units (rows or columns of an operand),
// packed as (E << 32) | float_bits(s): s = sum of (x / 2^(E-1023))^2 over one
// slab of the unit, E the slab's largest exponent field (zeros and subnormals
// contribute nothing).  FP32 with a running exponent keeps FP64 arithmetic, slow
// on GB300, out of the pass over the operands.  The partials of unit u are at
// p[u * unit_stride + i * part_stride], i < nparts.
struct StatParts {
    const unsigned long long *p;
    int n_units, nparts;
    long unit_stride, part_stride;
};

// Work items of the grouped stage-(a)/(b) launch (k_stage_jobs): each job is one
// of the per-problem kernels below, run on blocks [block0, block0 + gx * gy) of
// the launch with local block coordinates (bx, by).
enum StageKind : int { JOB_ROWMAX = 0, JOB_COLMAX = 1, JOB_SPLIT_A = 2, JOB_SPLIT_B = 3, JOB_STATS = 4 };
struct StageJob {
    int kind, gx, gy;
    const double *X;     // A (M x K) or B (K x N), row-major
    long ld;
    int rows, cols;      // of X
    int32_t *e_out;      // ROWMAX / COLMAX / STATS (rows): exponent fields, atomic max for STATS (may be null)
    double *ss_out;      // ROWMAX / COLMAX: sums of squares (may be null)
    const int32_t *e_in; // SPLIT: row (A) / column (B) exponents
    int b, s, KC, n_kc, padded, BN;  // SPLIT: padded = Mp (A) or Np (B)
    int f8;                          // SPLIT: e4m3 slices (b <= 4)
    int trans;                       // SPLIT: A stored K x M / B stored N x K
    uint16_t *tiles;
    int32_t *e_out2;                  // STATS: column exponent fields (atomic max, may be null)
    unsigned long long *prow, *pcol;  // STATS: row partials [rows][ceil(cols/256)], column partials [ceil(rows/64)][cols]
};
constexpr int kStageThreads = 256;
constexpr int kStatsCols = 256, kStatsRows = 64;  // STATS tile

// Per-problem inputs of the precision-knob reduction: the row exponents of op(A)
// and column exponents of op(B), and the partial sums of squares of the rows of
// op(A), columns of op(B), columns of op(A) and rows of op(B) (k units).
struct KnobJob {
    const int32_t *er;
    int M;
    const int32_t *ec;
    int N;
    int K;
    StatParts ra, cb, ka, kb;
    double *out;  // the 7 doubles of KnobStats (oz_plan.h), zeroed before
};

// Device error codes written to the error word.
enum DevErr : int { DEVERR_NONE = 0, DEVERR_TIMEOUT_PRODUCER = 1, DEVERR_TIMEOUT_MMA = 2, DEVERR_TIMEOUT_EPI = 3,
                    DEVERR_TIMEOUT_SELFTEST = 4 };

typedef void (*GemmLaunchFn)(const GemmArgs &args, int grid, size_t smem, void *stream);

// Kernel variants: (tile N, exact-accumulator words, K chunk).  Largest tile
// first; defined in oz_gemm_v*.cu.
#define OZ_GEMM_VARIANTS(X)                                                                        \
    X(128, 2, 32) X(128, 2, 16) X(64, 3, 32) X(64, 3, 16) X(64, 4, 32) X(64, 4, 16) X(48, 3, 32)   \
    X(48, 3, 16) X(48, 4, 32) X(48, 4, 16) X(32, 3, 32) X(32, 3, 16) X(32, 4, 32) X(32, 4, 16)     \
    X(32, 5, 32) X(32, 5, 16)                                                                       \
    X(16, 4, 32) X(16, 4, 16) X(16, 5, 32) X(16, 5, 16)
#define OZ_DECLARE_GEMM(BN, W, KC) void launch_gemm_##BN##_##W##_##KC(const GemmArgs &, int, size_t, void *);
OZ_GEMM_VARIANTS(OZ_DECLARE_GEMM)
// e4m3-carrier variants (b <= 4), KC in bf16-equivalent units (a 64-deep e4m3 chunk)
#define OZ_GEMM_F8_VARIANTS(X) \
    X(64, 3, 32) X(32, 3, 32) X(32, 4, 32) X(16, 4, 32) X(16, 5, 32) X(32, 3, 16) X(32, 4, 16) X(16, 4, 16) X(16, 5, 16)
#define OZ_DECLARE_GEMM_F8(BN, W, KC) void launch_gemm_f8_##BN##_##W##_##KC(const GemmArgs &, int, size_t, void *);
OZ_GEMM_F8_VARIANTS(OZ_DECLARE_GEMM_F8)

// Stage (a) / (b) launches (oz_split.cu).
void launch_rowmax(const double *A, long lda, int M, int K, int32_t *er, double *ss, void *stream);
void launch_colmax(const double *B, long ldb, int K, int N, int32_t *ec, double *ss, void *stream);
// trans: A is stored K x M (element (m, k) at A[k * lda + m]); B is stored N x K.
// f8: one-byte e4m3 slices (b <= 4), in the byte layout of a bf16 block of half the K chunk.
void launch_split_a(const double *A, long lda, int M, int K, const int32_t *er, int b, int s, int KC, int n_kc,
                    int Mp, uint16_t *tiles, void *stream, bool trans = false, bool f8 = false);
void launch_split_b(const double *B, long ldb, int K, int N, const int32_t *ec, int b, int s, int KC, int n_kc,
                    int BN, int Np, uint16_t *tiles, void *stream, bool trans = false, bool f8 = false);
int launch_selftest_timeout(int *err, unsigned long long timeout_ns, void *stream);
// Precision-knob statistics (seven doubles, KnobStats in oz_plan.h) of one
// problem; zeroes j.out first.
void launch_knob_stats(const KnobJob &j, void *stream);
// Grid sizes of the per-problem stage kernels (blocks in x and y of 256 threads).
void stage_grid(const StageJob &j, int *gx, int *gy);
// Grouped launches: all jobs in one grid (block0[i] = first block of job i,
// block0[n_jobs] = total), and the knob reduction of n problems.
void launch_stage_jobs(const StageJob *jobs, const int *block0, int n_jobs, int total_blocks, void *stream);
// Two jobs (for example the A and B halves of one stage) in one launch; the grid
// sizes are filled in here.
void launch_stage_pair(StageJob j0, StageJob j1, void *stream);
void launch_knob_grouped(const KnobJob *jobs, int n, void *stream);
// C = beta * C (zeros for beta == 0, C not read).
void launch_scale(double *C, long ldc, int M, int N, double beta, void *stream);
// Pseudo-random doubles in [-1, 1) for timing runs.
void launch_fill_random(double *x, size_t n, unsigned long long seed, void *stream);

}  // namespace ozgb
