// oz_plan.h -- host-side planning of one Ozaki DGEMM on GB300: slice/bin
// configuration, exact-accumulation limits, tile shape, bin blocks, pipeline depth.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "oz_internal.h"

namespace ozgb {

struct OzConfig {
    int b = 7;         // magnitude bits per slice
    int s = 8;         // slices
    int J = 8;         // bins: pair set {p + q <= J - 1}
    int rounding = 0;  // OUT_RN or OUT_RZ_REF
    int carrier = 0;   // 0: e4m3 slices where exact (b <= 4), else bf16; 1: bf16 (planes read back as bf16)
};

struct Plan {
    OzConfig cfg;
    int BN = 0, W = 0, KC = 0, stages = 0, G = 0, min_period = 0;  // KC: K values per chunk
    bool f8 = false;                  // e4m3 slices (kind::f8f6f4) instead of bf16
    size_t a_bytes = 0, b_bytes = 0;  // bytes of the slice blocks in HBM
    int n_kc = 0, Kp = 0, Mp = 0, Np = 0, tiles_m = 0, tiles_n = 0;
    int pairs = 0, max_pairs = 0, mma_per_kstep = 0;
    int pad_lo = 0, pad_hi = 0;
    size_t a_elems = 0, b_elems = 0;  // bf16 elements of the slice blocks in HBM
    uint32_t a_block_bytes = 0, b_block_bytes = 0, b_slice_bytes = 0, b_region_bytes = 0, stage_bytes = 0;
    uint32_t tmem_cols = 0;
    size_t smem = 0;
    double model_cycles_per_kstep = 0;  // UMMA cost model of the chosen blocks
    int blk_lo[kMaxGroups] = {0}, blk_nb[kMaxGroups] = {0}, blk_p0[kMaxGroups] = {0}, blk_p1[kMaxGroups] = {0};
    int blk_period[kMaxGroups] = {0}, blk_off[kMaxGroups] = {0};
    int n_acc = 0, acc_t0[kMaxAcc] = {0};  // drain accumulator groups (GemmArgs)
    int n_iss = 1;                         // MMA-issuing warps (1 to 3)
    uint32_t dbl_mask = 0;                 // double-buffered blocks (GemmArgs)
    int blk_col1[kMaxGroups] = {0};        // their second accumulator range (TMEM column)
    GemmLaunchFn fn = nullptr;
};

// Number of pairs (p, q), p, q < s, with p + q == j.
inline int pairs_in_bin(int j, int s) {
    const int lo = j - (s - 1) > 0 ? j - (s - 1) : 0;
    const int hi = j < s - 1 ? j : s - 1;
    return hi >= lo ? hi - lo + 1 : 0;
}

// Choices a plan may be forced to (0 = the planner's own choice): tile width BN,
// K chunk, number of bin blocks (the cheapest partition with exactly that many,
// or the explicit block sizes), pipeline stages.  The autotuner times
// candidates built from these.
struct PlanHints {
    int BN = 0, KC = 0, groups = 0, stages = 0;
    int sizes[kMaxGroups] = {0};  // explicit bin-block sizes (groups of them), overriding the cost model
    int min_W = 0;                // at least this many accumulator words (4 for OUT_PAIRS)
    int issuers = 0;              // MMA-issuing warps (1 to 3)
    int dbl = -1;                 // double-buffered blocks: -1 the planner's choice, 0 none, 1 every one that fits
};

// Builds the plan for bins [bin_lo, bin_hi] of the pair set (the full set of
// bins normally; a sub-range for parity dumps).  Returns false with a message
// when the configuration is outside the limits of the exact accumulation.  With
// no hints, a tuned entry for the problem's size class (tune_store) is used when
// one exists.
bool make_plan(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err, int bin_lo = 0,
               int bin_hi = 1 << 30, const PlanHints *hints = nullptr);

// Distinct feasible plans for the autotuner (at most max_n), the untuned plan first.
std::vector<PlanHints> plan_candidates(int M, int N, int K, const OzConfig &cfg, int max_n);

// Process-wide tuning table: the best hints per (bits, slices, bins, rounding,
// size class), the size class being ceil(log2) of M, N and K.
void tune_store(int M, int N, int K, const OzConfig &cfg, const PlanHints &h);
bool tune_lookup(int M, int N, int K, const OzConfig &cfg, PlanHints *h);
void tune_clear();
int tune_count();

// Bins in the reference's first (low-word) sum group, ozaki_base.cc:151-158 with
// log2 K = countr_zero(K) (include/oz_aie.h:100).
int reference_first_group(int K, int b, int d);

// The reference's (b, d) tables, include/oz_aie.h:60-80, indexed by log2 K.
void reference_table(int K, int mode, int *b, int *d);

// Precision-knob statistics, scaled by the largest row exponent ea of A and the
// largest column exponent eb of B:
//   sa = sum_i 4^{Er_i-ea},  na = ||A||_F^2 4^{1022-ea},
//   sb = sum_j 4^{Ec_j-eb},  nb = ||B||_F^2 4^{1022-eb},
//   t  = sum_k |A(:,k)|^2 |B(k,:)|^2 4^{2044-ea-eb}  (E||AB||_F^2 for random signs),
// and for the elementwise criterion the flattest row and column:
//   ia = max_i 1 / A_i,  A_i = |a_i|^2 4^{1022-Er_i}  (rows with a_i = 0 left out),
//   ib = max_j 1 / B_j,  B_j = |b_j|^2 4^{1022-Ec_j}.
// A_i is the sum of the squared magnitudes of row i scaled by its own largest
// element's power of two (each term < 1): about K/10 for a row of random
// magnitudes, 1/4 or less for a row that one element dominates.
struct KnobStats {
    double sa, na, sb, nb, t, ia, ib;
};

// Error criteria of the precision knob.
enum KnobCriterion : int { KNOB_NORMWISE = 0, KNOB_ELEMENTWISE = 1 };

// A-priori normwise relative error of the triangular pair set with s slices of
// b bits.  Write x = 2^{E-1022} (sum_p x_p 2^{-b(p+1)} + r 2^{-bs}) with digits
// x_p in [0, 2^b) and a truncated tail r in [0, 1).  For one product a b the
// error of the kept pairs p+q <= s-1 is 2^{Er+Ec-2044-bs} ((s-1)/4 + r_a beta +
// r_b alpha) to first order: the s-1 dropped pairs p+q = s (mean digit product
// 4^b/4, all of the product's sign) and the two tails (alpha, beta the scaled
// magnitudes).  Summing over k with random signs, over C, and bounding the
// three terms separately (Minkowski):
//   est(s) = 1.5 2^{-bs} ((s-1)/4 sqrt(K sa sb) + sqrt(sa nb / 3) + sqrt(sb na / 3)) / sqrt(t)
//            + 2^{-53} (rounding of the result).
// For phi <= 1 inputs the unscaled model is within a few percent of the
// measured error; heavier tails make it conservative.  Non-finite or zero
// statistics give an infinite estimate (the caller then takes its largest s).
//
// Elementwise criterion (crit = KNOB_ELEMENTWISE): the relative error of each
// entry c_ij with |c_ij| >= tail h_ij, h_ij = |a_i| |b_j| / sqrt(K) the rms
// scale of the entry's K terms.  Per entry the same first-order terms, summed
// with random signs, give |e_ij| / h_ij = 2^{-bs} sqrt(K) sqrt(K (s-1)^2 /
// (16 A_i B_j) + 1 / (3 A_i) + 1 / (3 B_j)) (h_ij = 2^{Er_i+Ec_j-2044}
// sqrt(A_i B_j / K) exactly); the flattest row and column (ia, ib) bound it over
// all entries:
//   est_e(s) = 4 2^{-bs} sqrt(K) sqrt(K (s-1)^2 ia ib / 16 + (ia + ib) / 3) / tail + 2^{-53}
// (the factor 4: the largest of many entries' errors is about 4 of their
// standard deviations).
// No fixed precision bounds the relative error of an entry that cancels to
// near zero; the tail leaves out the entries within tail h_ij of zero (about a
// tail's fraction of them for random signs and phi <= 1; more for heavy tails,
// whose few large terms make h_ij large against most entries).
double knob_estimate(const KnobStats &k, int K, int b, int s, int crit = KNOB_NORMWISE, double tail = 1e-4);

// The same for the pair set p + q <= J - 1, s <= J <= 2s - 1 (J = s: the
// triangular set above).  The first dropped pairs are then those with p + q = J,
// pairs_in_bin(J, s) of them, each of weight 2^{-bJ}/4 on average, so the first
// term becomes pairs_in_bin(J, s)/4 2^{-bJ} sqrt(K sa sb) (elementwise: likewise
// inside the square root), while the truncated tails stay at 2^{-bs}.  With the
// full set (J = 2s - 1) only the tails remain.
double knob_estimate_set(const KnobStats &k, int K, int b, int s, int J, int crit = KNOB_NORMWISE,
                         double tail = 1e-4);

// A slice schedule: slices s and pair set J, with its estimate and modelled time.
struct Schedule {
    int s = 0, J = 0;
    double est = 0.0, ms = 0.0;
};

// Modelled time (ms) of one M x N x K product with a plan on `sms` SMs: the
// plan's modelled SM cycles per K step (model_cycles_per_kstep, the bin-block cost
// model fitted to the slice-pair GEMM on GB300) at 2 GHz, over whole waves of
// tiles, plus the HBM traffic of the split at 6.5 TB/s.
double plan_time_model(const Plan &p, int M, int N, int K, int sms);

// The slice schedule for a requested bound: among s in [s_min, s_max] and, with
// any_set, every pair set J in [s, 2s - 1] (else J = s only), the one with the
// smallest modelled time whose estimate meets the bound (ties: fewer slices,
// then fewer bins).  For each s only the smallest J that meets the bound is a
// candidate (a larger J only adds pairs).  With none meeting it: (s_max, s_max).
// Without any_set: the fewest slices s with J = s that meet the bound
// (choose_slices_stats).
Schedule choose_schedule(const KnobStats &k, int M, int N, int K, const OzConfig &base, double bound, int s_min,
                         int s_max, int crit, double tail, bool any_set, int sms);

// Slice count for a requested relative error: the smallest s in [s_min, s_max]
// with knob_estimate <= bound (s_max if none).  Writes the estimate for the
// returned s.
int choose_slices_stats(const KnobStats &k, int K, int b, double bound, int s_min, int s_max, double *estimate,
                        int crit = KNOB_NORMWISE, double tail = 1e-4);

// KnobStats computed on the host from stage-(a) style statistics.  ca/rb (the
// per-k sums of squares of the columns of A and the rows of B) may be null:
// t then falls back to ||A||^2 ||B||^2 / K (mass spread evenly over k).
KnobStats knob_stats_host(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                          const double *ca, const double *rb, int K);

}  // namespace ozgb
