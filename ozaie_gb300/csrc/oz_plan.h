// oz_plan.h -- host-side planning of one Ozaki DGEMM on GB300: slice/bin
// configuration, exact-accumulation limits, tile shape, bin blocks, pipeline depth.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include "oz_internal.h"

namespace ozgb {

struct OzConfig {
    int b = 7;         // magnitude bits per slice
    int s = 8;         // slices
    int J = 8;         // bins: pair set {p + q <= J - 1}
    int rounding = 0;  // OUT_RN or OUT_RZ_REF
};

struct Plan {
    OzConfig cfg;
    int BN = 0, W = 0, KC = 0, stages = 0, G = 0, min_period = 0;
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
    GemmLaunchFn fn = nullptr;
};

// Number of pairs (p, q), p, q < s, with p + q == j.
inline int pairs_in_bin(int j, int s) {
    const int lo = j - (s - 1) > 0 ? j - (s - 1) : 0;
    const int hi = j < s - 1 ? j : s - 1;
    return hi >= lo ? hi - lo + 1 : 0;
}

// Builds the plan for bins [bin_lo, bin_hi] of the pair set (the full set of
// bins normally; a sub-range for parity dumps).  Returns false with a message
// when the configuration is outside the limits of the exact accumulation.
bool make_plan(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err, int bin_lo = 0,
               int bin_hi = 1 << 30);

// The reference's (b, d) tables, include/oz_aie.h:60-80, indexed by log2 K.
void reference_table(int K, int mode, int *b, int *d);

// Slice count for a requested normwise relative error, from the stage-(a)
// statistics (max exponents and sums of squares).  Returns the chosen s and
// writes the a-priori estimate for it.
int choose_slices(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N, int K,
                  int b, double bound, int s_min, int s_max, double *estimate);
// The same rule from the two spread factors rho_A, rho_B (computed on the device
// by launch_knob_rho, or on the host by choose_slices).
int choose_slices_rho(double ra, double rb, int b, double bound, int s_min, int s_max, double *estimate);

}  // namespace ozgb
