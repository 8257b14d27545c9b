// oz_plan.cpp -- planning of the GB300 Ozaki DGEMM (host only, no CUDA calls).
#include "oz_plan.h"

#include <algorithm>
#include <cmath>

namespace ozgb {

namespace {

struct Variant {
    int BN, W;
    GemmLaunchFn fn;
};

// Kernel variants, largest tile first.  BN * J <= 512 TMEM columns and the
// drain registers (BN/2 * W words) bound which ones exist.
const Variant kVariants[] = {
    {128, 2, launch_gemm_128_2}, {64, 3, launch_gemm_64_3}, {64, 4, launch_gemm_64_4},
    {48, 3, launch_gemm_48_3},   {48, 4, launch_gemm_48_4}, {32, 4, launch_gemm_32_4},
    {32, 5, launch_gemm_32_5},   {16, 4, launch_gemm_16_4}, {16, 5, launch_gemm_16_5},
};

constexpr size_t kSmemLimit = 232448;  // max dynamic shared memory per block on sm_103
constexpr size_t kSmemReserve = 2048 + 1024;

}  // namespace

void reference_table(int K, int mode, int *b, int *d) {
    // include/oz_aie.h:60-80; the reference only reaches log2 K in [7, 11], the
    // table lists up to 14 and is clamped at both ends here.
    static const int acc_b[8] = {3, 3, 3, 3, 3, 3, 3, 4};
    static const int acc_d[8] = {29, 28, 27, 27, 26, 25, 25, 18};
    int l2 = 0;
    while ((2 << l2) <= K) ++l2;  // floor(log2 K) for K >= 1
    int idx = std::min(std::max(l2 - 7, 0), 7);
    if (mode == 0) {
        *b = acc_b[idx];
        *d = acc_d[idx];
    } else {
        *b = 7;
        *d = 8;
    }
}

bool make_plan(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err) {
    Plan p;
    p.cfg = cfg;
    const int b = cfg.b, s = cfg.s, J = cfg.J;
    if (M < 1 || N < 1 || K < 1) {
        *err = "dimensions must be positive";
        return false;
    }
    if (b < 1 || b > 7) {
        *err = "bits per slice must be in [1, 7] (slices are int8 with a sign)";
        return false;
    }
    if (s < 1 || J < 1 || J > 2 * s - 1 || J > 32) {
        *err = "need 1 <= bins <= min(2*slices-1, 32)";
        return false;
    }
    {
        // the split keeps at most 128 - (bits shifted out) bits of the aligned mantissa
        const int avoid = 1 + (b == 3 ? 3 : 0);
        const int nv0 = 64 - avoid - ((64 - avoid) % b);
        const int cap = (s * b <= nv0) ? nv0 : nv0 + (64 - avoid);
        if (s * b > cap) {
            *err = "slices * bits exceeds the split window";
            return false;
        }
    }
    const double v2 = std::ldexp(1.0, b) - 1.0;
    p.pairs = 0;
    p.max_pairs = 0;
    long double bound = 0.0L;
    for (int j = 0; j < J; ++j) {
        const int pj = pairs_in_bin(j, s);
        p.pairs += pj;
        p.max_pairs = std::max(p.max_pairs, pj);
        bound += std::ldexp(static_cast<long double>(pj) * v2 * v2 * K, b * (J - 1 - j));
    }
    const int bits = static_cast<int>(std::ceil(std::log2(static_cast<double>(bound) + 1.0))) + 1;
    // K values a bin may accumulate in fp32 between drains: every partial sum
    // stays an integer of magnitude <= 2^24.
    const long kb_max = static_cast<long>(std::floor(16777216.0 / (p.max_pairs * v2 * v2)));
    if (kb_max < 16) {
        *err = "too many pairs per bin for exact fp32 accumulation of one 16-deep K step";
        return false;
    }
    const Variant *chosen = nullptr;
    for (const Variant &v : kVariants) {
        if (v.BN * J > 512) continue;
        if (32 * v.W < bits) continue;
        chosen = &v;
        break;
    }
    if (!chosen) {
        *err = "no kernel variant holds " + std::to_string(J) + " bins with a " + std::to_string(bits) +
               "-bit exact accumulator";
        return false;
    }
    p.BN = chosen->BN;
    p.W = chosen->W;
    p.fn = chosen->fn;

    const size_t budget = kSmemLimit - kSmemReserve;
    const int kc_opts[3] = {64, 32, 16};
    p.KC = 0;
    for (int kc : kc_opts) {
        if (kc > kb_max) continue;
        if (kc > 16 && kc > ((K + 15) / 16) * 16) continue;  // no wider than K needs
        const size_t stage = static_cast<size_t>(s) * (BM + p.BN) * kc * 2;
        const size_t st = budget / stage;
        if (st >= 2) {
            p.KC = kc;
            p.stages = static_cast<int>(std::min<size_t>(st, 8));
            break;
        }
    }
    if (!p.KC) {
        const size_t stage = static_cast<size_t>(s) * (BM + p.BN) * 16 * 2;
        if (stage > budget) {
            *err = "slices do not fit one 16-deep pipeline stage in shared memory";
            return false;
        }
        p.KC = 16;
        p.stages = 1;
    }
    p.n_kc = (K + p.KC - 1) / p.KC;
    p.Kp = p.n_kc * p.KC;
    p.KBc = std::max(1, static_cast<int>(kb_max / p.KC));
    if (p.n_kc <= p.KBc) {
        p.G = 1;  // no drain before the last chunk
    } else {
        p.G = std::min(J, p.KBc);
    }
    if (p.G > kMaxGroups) p.G = kMaxGroups;
    for (int g = 0; g < p.G; ++g) {
        p.grp_lo[g] = (g * J) / p.G;
        p.grp_hi[g] = ((g + 1) * J) / p.G - 1;
    }
    p.tiles_m = (M + BM - 1) / BM;
    p.tiles_n = (N + p.BN - 1) / p.BN;
    p.Mp = p.tiles_m * BM;
    p.Np = p.tiles_n * p.BN;
    p.a_block_bytes = static_cast<uint32_t>(s) * BM * p.KC * 2;
    p.b_block_bytes = static_cast<uint32_t>(s) * p.BN * p.KC * 2;
    p.stage_bytes = p.a_block_bytes + p.b_block_bytes;
    p.a_elems = static_cast<size_t>(p.tiles_m) * p.n_kc * s * BM * p.KC;
    p.b_elems = static_cast<size_t>(p.tiles_n) * p.n_kc * s * p.BN * p.KC;
    uint32_t cols = 32;
    while (cols < static_cast<uint32_t>(J * p.BN)) cols <<= 1;
    p.tmem_cols = cols;
    p.smem = static_cast<size_t>(p.stages) * p.stage_bytes + 1024 + 2048;
    *out = p;
    return true;
}

int choose_slices(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N, int K,
                  int b, double bound, int s_min, int s_max, double *estimate) {
    // Dropped pairs p + q = s dominate the error of the triangular set: each is a
    // product of two digits of rms ~0.57 * 2^b at weights 2^{E-1022-b(p+1)}, summed
    // over s-1 pairs with random signs.  The truncated tails add ~0.58 2^{-bs} per
    // operand.  Relative to the rms size of C this gives, with
    // rho_A^2 = sum_i 4^{Er_i-1022} / sum_i (|a_i|^2 / K) and rho_B likewise,
    //   est(s) = 2^{-bs} (0.33 sqrt(s-1) rho_A rho_B + 0.58 (rho_A + rho_B)).
    auto rho = [K](const int32_t *e, const double *ss, int n) {
        int emax = 0;
        for (int i = 0; i < n; ++i) emax = std::max(emax, static_cast<int>(e[i]));
        long double num = 0.0L, den = 0.0L;
        for (int i = 0; i < n; ++i) {
            num += std::ldexp(1.0L, 2 * (e[i] - emax));
            den += std::ldexp(static_cast<long double>(ss[i]) / K, -2 * (emax - 1022));
        }
        if (den <= 0.0L) return 1.0;
        return static_cast<double>(std::sqrt(num / den));
    };
    const double ra = rho(er, ssr, M), rb = rho(ec, ssc, N);
    const double safety = 2.0;
    int s = s_min;
    double est = 0.0;
    for (s = s_min; s <= s_max; ++s) {
        est = safety * std::ldexp(0.33 * std::sqrt(std::max(1.0, s - 1.0)) * ra * rb + 0.58 * (ra + rb), -b * s);
        if (est <= bound) break;
    }
    if (s > s_max) s = s_max;
    if (estimate) *estimate = est;
    return s;
}

}  // namespace ozgb
