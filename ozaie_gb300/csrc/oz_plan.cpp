// oz_plan.cpp -- planning of the GB300 Ozaki DGEMM (host only, no CUDA calls).
#include "oz_plan.h"

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <unordered_map>
#include <vector>

namespace ozgb {

namespace {

struct Variant {
    int BN, W, KC;  // KC: the kernel's chunk in bf16-equivalent units (K values for bf16, half of them for e4m3)
    bool f8;
    GemmLaunchFn fn;
};

#define OZ_VARIANT_ENTRY(BN, W, KC) {BN, W, KC, false, launch_gemm_##BN##_##W##_##KC},
#define OZ_VARIANT_ENTRY_F8(BN, W, KC) {BN, W, KC, true, launch_gemm_f8_##BN##_##W##_##KC},
// Kernel variants, largest tile first.  BN * J <= 512 TMEM columns and the
// drain registers (2 (W-1) words per column) bound which ones exist.
const Variant kVariants[] = {OZ_GEMM_VARIANTS(OZ_VARIANT_ENTRY) OZ_GEMM_F8_VARIANTS(OZ_VARIANT_ENTRY_F8)};

constexpr size_t kSmemLimit = 232448;  // max dynamic shared memory per block on sm_103
constexpr size_t kSmemReserve = kCtrlBytes;

}  // namespace

int reference_first_group(int K, int b, int d) {
    int ctz = 0;
    while (ctz < 31 && !((K >> ctz) & 1)) ++ctz;
    const int alignable = 31 / b + 1;
    const int numer = b * (d + 1) - 51 + ctz;
    const int minfirst = numer < 0 ? 1 : numer / b + 1;
    return std::min(d, std::max(minfirst, alignable));
}

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

namespace {
using TuneKey = std::tuple<int, int, int, int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<TuneKey, PlanHints> g_tune;
long g_tune_generation = 0;  // bumped whenever the table changes (plans cached under the old one are stale)

int ceil_log2(int x) {
    int l = 0;
    while ((1L << l) < x) ++l;
    return l;
}
TuneKey tune_key(int M, int N, int K, const OzConfig &cfg) {
    return TuneKey{cfg.b, cfg.s, cfg.J, cfg.rounding, cfg.carrier, ceil_log2(M), ceil_log2(N), ceil_log2(K)};
}
}  // namespace

void tune_store(int M, int N, int K, const OzConfig &cfg, const PlanHints &h) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(M, N, K, cfg)] = h;
    ++g_tune_generation;
}
bool tune_lookup(int M, int N, int K, const OzConfig &cfg, PlanHints *h) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(M, N, K, cfg));
    if (it == g_tune.end()) return false;
    *h = it->second;
    return true;
}
void tune_clear() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
    ++g_tune_generation;
}
int tune_count() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return static_cast<int>(g_tune.size());
}

namespace {
bool make_plan_uncached(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err, int bin_lo, int bin_hi,
                        const PlanHints *hints);
}

namespace {
// Plans without hints are pure functions of the shape, the configuration and the
// tuning table: cached, so that grouped calls with many problems plan in O(1) each.
using PlanKey = std::tuple<int, int, int, int, int, int, int, int, int, int, long>;
struct PlanKeyHash {
    size_t operator()(const PlanKey &k) const {
        const long long v[11] = {std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k),
                                 std::get<4>(k), std::get<5>(k), std::get<6>(k), std::get<7>(k),
                                 std::get<8>(k), std::get<9>(k), std::get<10>(k)};
        unsigned long long h = 1469598103934665603ull;  // FNV-1a
        for (long long x : v) h = (h ^ static_cast<unsigned long long>(x)) * 1099511628211ull;
        return static_cast<size_t>(h);
    }
};
std::mutex g_plan_mu;
std::unordered_map<PlanKey, Plan, PlanKeyHash> g_plans;
}  // namespace

bool make_plan(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err, int bin_lo, int bin_hi,
               const PlanHints *hints) {
    if (hints)
        return make_plan_uncached(M, N, K, cfg, out, err, bin_lo, bin_hi, hints);
    long gen;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        gen = g_tune_generation;
    }
    const PlanKey key{M, N, K, cfg.b, cfg.s, cfg.J, cfg.rounding, cfg.carrier, bin_lo, std::min(bin_hi, 1 << 20), gen};
    {
        std::lock_guard<std::mutex> lk(g_plan_mu);
        auto it = g_plans.find(key);
        if (it != g_plans.end()) {
            *out = it->second;
            return true;
        }
    }
    Plan p;
    if (!make_plan_uncached(M, N, K, cfg, &p, err, bin_lo, bin_hi, nullptr)) return false;
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (g_plans.size() > 8192) g_plans.clear();
    g_plans[key] = p;
    *out = p;
    return true;
}

namespace {
bool make_plan_uncached(int M, int N, int K, const OzConfig &cfg, Plan *out, std::string *err, int bin_lo, int bin_hi,
                        const PlanHints *hints) {
    PlanHints tuned;
    if (!hints && bin_lo <= 0 && bin_hi >= cfg.J - 1 && tune_lookup(M, N, K, cfg, &tuned)) hints = &tuned;
    const PlanHints none;
    const PlanHints &hint = hints ? *hints : none;
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
    const int B0 = std::max(0, bin_lo), B1 = std::min(J - 1, bin_hi);
    if (B0 > B1) {
        *err = "empty bin range";
        return false;
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
    // stays an integer of magnitude <= 2^24 (tightest bin).
    const long kb_max = static_cast<long>(std::floor(16777216.0 / (p.max_pairs * v2 * v2)));
    if (kb_max < 16) {
        *err = "too many pairs per bin for exact fp32 accumulation of one 16-deep K step";
        return false;
    }
    // Drain accumulator groups: consecutive t = J - 1 - j (increasing weight) share
    // one 64-bit accumulator while the weight relative to the group's first bin
    // stays <= 2^30 (one 32 x 32 -> 64-bit multiply-add per drained value) and the
    // group's worst-case sum over all of K stays below 2^62.
    int n_acc = 0, acc_t0[kMaxAcc] = {0};
    {
        long double gsum = 0.0L;
        int t0 = 0;
        for (int t = 0; t < J; ++t) {
            const long double one = static_cast<long double>(pairs_in_bin(J - 1 - t, s)) * v2 * v2 * K;
            const int rel = b * (t - t0);
            const long double add = std::ldexp(one, rel);
            if (n_acc > 0 && rel <= 30 && gsum + add < std::ldexp(1.0L, 62)) {
                gsum += add;
                continue;
            }
            if (n_acc == kMaxAcc) {
                *err = "the exact accumulation needs more than " + std::to_string(kMaxAcc) + " 64-bit groups";
                return false;
            }
            acc_t0[n_acc++] = t;
            t0 = t;
            gsum = one;
        }
    }
    // Carrier: e4m3 holds every slice of b <= 4 bits (|v| <= 15) exactly and one
    // kind::f8f6f4 UMMA covers 32 K values, twice a bf16 UMMA's, for about the same
    // time; bf16 otherwise, or when the planes are read back as bf16.
    auto pick = [&](bool f8) -> const Variant * {
        for (const Variant &v : kVariants) {
            if (v.f8 != f8 || v.KC != 32) continue;
            if (hint.BN && v.BN != hint.BN) continue;
            if (v.W < hint.min_W) continue;
            if (std::max(1, v.W - 1) < n_acc) continue;  // accumulator groups the variant holds
            if (v.BN * J > 512) continue;
            if (32 * v.W < bits) continue;
            return &v;
        }
        return nullptr;
    };
    const Variant *chosen = (b <= 4 && cfg.carrier != 1 && kb_max >= 64) ? pick(true) : nullptr;
    p.f8 = chosen != nullptr;
    if (!chosen) chosen = pick(false);
    if (!chosen) {
        *err = "no kernel variant holds " + std::to_string(J) + " bins with a " + std::to_string(bits) +
               "-bit exact accumulator";
        return false;
    }
    p.BN = chosen->BN;
    p.W = chosen->W;
    p.n_acc = n_acc;
    for (int a = 0; a < kMaxAcc; ++a) p.acc_t0[a] = acc_t0[a];

    // ---- bin blocks: contiguous bin ranges of at most 256 columns; every UMMA of a
    // block spans the whole block (zero B slices pad the out-of-range q).  Cost of
    // a partition per 16-deep K step of a tile, in SM cycles, fitted to GB300
    // measurements of the kernel (three issuing warps, tests/perf/umma_cost.cu for
    // the UMMA itself): each UMMA N / 2 + 20 (the tensor pipe takes half a cycle per
    // column; the A tile is re-read from shared memory for every UMMA), each block
    // 200 (per-block issue work), and for each block the part of its drain (500 +
    // 800 per 48 columns: the F2I conversions run at 16 per cycle per SM) that two
    // K steps of the other blocks' UMMAs do not cover, once per drain period.  The
    // search enumerates the compositions of the bins into G <= 8 blocks whose sizes
    // stay within one of the even split, for every G.
    const int max_groups = kMaxGroups;
    const int maxb = 256 / p.BN;
    const int kpu = p.f8 ? 32 : 16;  // K values per UMMA
    auto p0_of = [s](int lo) { return std::max(0, lo - (s - 1)); };
    auto p1_of = [s](int hi) { return std::min(hi, s - 1); };
    auto period_k = [&](int lo, int nb) {  // K values a block accumulates between drains
        long kb = 1L << 40;
        for (int j = lo; j < lo + nb; ++j)
            if (pairs_in_bin(j, s) > 0)
                kb = std::min(kb, static_cast<long>(std::floor(16777216.0 / (pairs_in_bin(j, s) * v2 * v2))));
        const long chunk = 2L * kpu;  // a pipeline chunk holds two UMMA K steps
        return std::max(chunk, (kb / chunk) * chunk);
    };
    auto part_cost = [&](int G, const int *lo, const int *nb) {
        double t[kMaxGroups], T = 200.0 * G;
        for (int g = 0; g < G; ++g) {
            const int runs = p1_of(lo[g] + nb[g] - 1) - p0_of(lo[g]) + 1;
            t[g] = runs * (0.5 * nb[g] * p.BN + 20.0);
            T += t[g];
        }
        double stall = 0.0;
        for (int g = 0; g < G; ++g) {
            const double drain = 500.0 + 800.0 * nb[g] * p.BN / 48.0;
            stall += std::max(0.0, drain - 2.0 * (T - t[g])) * kpu / static_cast<double>(period_k(lo[g], nb[g]));
        }
        return T + stall;
    };
    const int nbins = B1 - B0 + 1;
    double best_cost = HUGE_VAL;
    int best_G = 0, best_nb[kMaxGroups] = {0};
    const bool explicit_sizes = hint.groups && hint.sizes[0] > 0;
    if (!explicit_sizes) {
        int nb[kMaxGroups], lo[kMaxGroups];
        // sizes of block g .. G-1 for bins at .. B1, each in [smin, smax]
        std::function<void(int, int, int, int, int)> rec = [&](int g, int at, int G, int smin, int smax) {
            if (g == G) {
                if (at != B1 + 1) return;
                const double c = part_cost(G, lo, nb);
                if (c < best_cost - 1e-9) {
                    best_cost = c;
                    best_G = G;
                    for (int i = 0; i < G; ++i) best_nb[i] = nb[i];
                }
                return;
            }
            const int left = B1 + 1 - at, rest = G - g - 1;
            for (int sz = smin; sz <= smax; ++sz) {
                if (sz > left || left - sz < rest * smin || left - sz > rest * smax) continue;
                lo[g] = at;
                nb[g] = sz;
                rec(g + 1, at + sz, G, smin, smax);
            }
        };
        for (int G = 1; G <= std::min(max_groups, nbins); ++G) {
            if (hint.groups && G != hint.groups) continue;
            if ((nbins + G - 1) / G > maxb) continue;
            const int smin = std::max(1, nbins / G - 1), smax = std::min(maxb, (nbins + G - 1) / G + 1);
            rec(0, B0, G, smin, smax);
        }
    }
    if (!best_G && !explicit_sizes) {
        *err = "bins do not fit " + std::to_string(max_groups) + " blocks of at most 256 columns";
        return false;
    }
    p.G = best_G;
    p.model_cycles_per_kstep = best_cost;
    for (int g = 0, at = B0; g < p.G; at += best_nb[g], ++g) {
        p.blk_lo[g] = at;
        p.blk_nb[g] = best_nb[g];
    }
    if (explicit_sizes) {
        // explicit block sizes: contiguous, covering the bins, each at most 256 columns
        int at = B0;
        for (int g = 0; g < hint.groups; ++g) {
            const int nb = hint.sizes[g];
            if (nb < 1 || nb > maxb || at + nb - 1 > B1) {
                *err = "hinted bin blocks do not fit";
                return false;
            }
            p.blk_lo[g] = at;
            p.blk_nb[g] = nb;
            at += nb;
        }
        if (at != B1 + 1) {
            *err = "hinted bin blocks do not cover the bins";
            return false;
        }
        p.G = hint.groups;
        p.model_cycles_per_kstep = part_cost(p.G, p.blk_lo, p.blk_nb);
    }
    p.pad_lo = 0;
    p.pad_hi = 0;
    p.mma_per_kstep = 0;
    for (int g = 0; g < p.G; ++g) {
        const int lo = p.blk_lo[g], hi = lo + p.blk_nb[g] - 1;
        p.blk_p0[g] = p0_of(lo);
        p.blk_p1[g] = p1_of(hi);
        p.mma_per_kstep += p.blk_p1[g] - p.blk_p0[g] + 1;
        p.pad_lo = std::max(p.pad_lo, p.blk_p1[g] - lo);           // q = lo - p1 >= -pad_lo
        p.pad_hi = std::max(p.pad_hi, hi - p.blk_p0[g] - (s - 1));  // q = hi - p0 <= s - 1 + pad_hi
    }

    // issuing warps (1 to 3; the UMMA runs of a K step are dealt round-robin): one
    // warp issues a UMMA about every 80-100 SM cycles and the tensor pipe takes
    // N / 2 cycles for N columns, so three unless there are fewer runs than that
    p.n_iss = hint.issuers >= 1 && hint.issuers <= kMaxIssuers ? hint.issuers : kMaxIssuers;
    p.n_iss = std::min(p.n_iss, std::max(1, p.mma_per_kstep));

    // ---- pipeline: K chunk and stage count (a chunk of 32 bf16 or 64 e4m3 K values
    // is 64 bytes per row and slice)
    const size_t eb = p.f8 ? 1 : 2;
    const size_t budget = kSmemLimit - kSmemReserve;
    const int kc_opts[2] = {p.f8 ? 64 : 32, p.f8 ? 32 : 16};
    const int kmin = kc_opts[1];
    const int force_kc = hint.KC;
    auto stage_of = [&](int kc) {
        return (static_cast<size_t>(s) * BM * kc + static_cast<size_t>(p.pad_lo + s + p.pad_hi) * p.BN * kc) * eb;
    };
    p.KC = 0;
    for (int kc : kc_opts) {
        if (force_kc && kc != force_kc) continue;
        if (kc > kb_max) continue;
        if (kc > kmin && kc > ((K + kmin - 1) / kmin) * kmin) continue;  // no wider than K needs
        const size_t st = budget / stage_of(kc);
        if (st >= 2) {
            p.KC = kc;
            p.stages = static_cast<int>(std::min<size_t>(st, 8));
            if (hint.stages >= 2) p.stages = std::min(p.stages, hint.stages);
            break;
        }
    }
    if (!p.KC) {
        if (stage_of(kmin) > budget) {
            *err = "slices do not fit one pipeline stage in shared memory";
            return false;
        }
        p.KC = kmin;
        p.stages = 1;
    }
    p.fn = nullptr;
    const int vkc = p.f8 ? p.KC / 2 : p.KC;  // the kernel's bf16-equivalent chunk
    for (const Variant &v : kVariants)
        if (v.f8 == p.f8 && v.BN == p.BN && v.W == p.W && v.KC == vkc) p.fn = v.fn;
    if (!p.fn && p.f8) {
        // no e4m3 kernel for this tile / accumulator / chunk: the same with bf16 slices
        OzConfig c2 = cfg;
        c2.carrier = 1;
        return make_plan_uncached(M, N, K, c2, out, err, bin_lo, bin_hi, hints);
    }
    if (!p.fn) {
        *err = "no kernel variant for this tile / accumulator / K chunk";
        return false;
    }
    p.n_kc = (K + p.KC - 1) / p.KC;
    p.Kp = p.n_kc * p.KC;

    // ---- drain periods: bin j may accumulate KB_j K-values in fp32 with
    // pairs_j * KB_j * (2^b-1)^2 <= 2^24; a block drains at its tightest bin's
    // period (in chunks).  A period >= n_kc means only after the last chunk.
    // Periods and offsets do not depend on K (a period longer than a tile's chunks
    // only drains at the tile's end), so problems of one shape class share a plan.
    p.min_period = 1 << 20;
    for (int g = 0; g < p.G; ++g) {
        int per = 1 << 20;
        for (int j = p.blk_lo[g]; j < p.blk_lo[g] + p.blk_nb[g]; ++j) {
            const long kbj = static_cast<long>(std::floor(16777216.0 / (pairs_in_bin(j, s) * v2 * v2)));
            per = std::min<long>(per, std::max(1L, kbj / p.KC));
        }
        p.blk_period[g] = per;
        p.min_period = std::min(p.min_period, per);
    }
    // stagger the drains of different blocks across chunks
    for (int g = 0; g < p.G; ++g) p.blk_off[g] = (g * p.blk_period[g]) / std::max(1, p.G);

    p.tiles_m = (M + BM - 1) / BM;
    p.tiles_n = (N + p.BN - 1) / p.BN;
    p.Mp = p.tiles_m * BM;
    p.Np = p.tiles_n * p.BN;
    p.b_slice_bytes = static_cast<uint32_t>(p.BN * p.KC * eb);
    p.a_block_bytes = static_cast<uint32_t>(s * BM * p.KC * eb);
    p.b_block_bytes = static_cast<uint32_t>(s) * p.b_slice_bytes;
    p.b_region_bytes = static_cast<uint32_t>(p.pad_lo + s + p.pad_hi) * p.b_slice_bytes;
    p.stage_bytes = p.a_block_bytes + p.b_region_bytes;
    p.a_elems = static_cast<size_t>(p.tiles_m) * p.n_kc * s * BM * p.KC;
    p.b_elems = static_cast<size_t>(p.tiles_n) * p.n_kc * s * p.BN * p.KC;
    p.a_bytes = p.a_elems * eb;
    p.b_bytes = p.b_elems * eb;
    // ---- double buffering: blocks get a second accumulator range in the TMEM
    // columns the bins leave free, most frequently drained blocks first (the
    // order does not depend on K, so problems of one shape class share a plan);
    // their UMMAs then switch ranges at each drain, and at the end of a tile,
    // instead of waiting for the drain warps to read the block out.
    p.dbl_mask = 0;
    int next_col = J * p.BN;  // buffer 0: bin j at column j BN
    if (hint.dbl != 0) {
        int order[kMaxGroups], n = 0;
        long period[kMaxGroups];  // in K values, not clamped to this K
        for (int g = 0; g < p.G; ++g) {
            order[n++] = g;
            period[g] = 1L << 40;
            for (int j = p.blk_lo[g]; j < p.blk_lo[g] + p.blk_nb[g]; ++j)
                period[g] = std::min(period[g], static_cast<long>(std::floor(16777216.0 / (pairs_in_bin(j, s) * v2 * v2))));
        }
        std::sort(order, order + n, [&](int x, int y) {
            return period[x] != period[y] ? period[x] < period[y] : (p.blk_nb[x] != p.blk_nb[y] ? p.blk_nb[x] > p.blk_nb[y] : x < y);
        });
        for (int i = 0; i < n; ++i) {
            const int g = order[i];
            if (next_col + p.blk_nb[g] * p.BN > 512) continue;
            p.dbl_mask |= 1u << g;
            p.blk_col1[g] = next_col;
            next_col += p.blk_nb[g] * p.BN;
        }
    }
    uint32_t cols = 32;
    while (cols < static_cast<uint32_t>(next_col)) cols <<= 1;
    p.tmem_cols = cols;
    p.smem = static_cast<size_t>(p.stages) * p.stage_bytes + kCtrlBytes;
    *out = p;
    return true;
}

}  // namespace

std::vector<PlanHints> plan_candidates(int M, int N, int K, const OzConfig &cfg, int max_n) {
    std::vector<PlanHints> out;
    std::vector<Plan> plans;
    auto same = [](const Plan &x, const Plan &y) {
        if (x.f8 != y.f8 || x.BN != y.BN || x.KC != y.KC || x.G != y.G || x.stages != y.stages ||
            x.n_iss != y.n_iss || x.dbl_mask != y.dbl_mask)
            return false;
        for (int i = 0; i < x.G; ++i)
            if (x.blk_lo[i] != y.blk_lo[i] || x.blk_nb[i] != y.blk_nb[i]) return false;
        return true;
    };
    auto try_add = [&](const PlanHints &h) {
        Plan p;
        std::string why;
        if (!make_plan(M, N, K, cfg, &p, &why, 0, 1 << 30, &h)) return;
        for (const Plan &q : plans)
            if (same(p, q)) return;
        PlanHints exact = h;
        exact.BN = p.BN;
        exact.KC = p.KC;
        exact.groups = p.G;
        exact.stages = p.stages;
        exact.issuers = p.n_iss;
        exact.dbl = p.dbl_mask ? 1 : 0;
        for (int g = 0; g < kMaxGroups; ++g) exact.sizes[g] = g < p.G ? p.blk_nb[g] : 0;
        plans.push_back(p);
        out.push_back(exact);
        if (!h.issuers) {
            // the same plan with fewer issuing warps
            for (int ni = p.n_iss - 1; ni >= 1; --ni) {
                PlanHints fewer = exact;
                fewer.issuers = ni;
                Plan q;
                if (make_plan(M, N, K, cfg, &q, &why, 0, 1 << 30, &fewer)) {
                    plans.push_back(q);
                    out.push_back(fewer);
                }
            }
        }
    };
    try_add(PlanHints{});  // the cost-model choice
    const int bns[] = {128, 64, 48, 32, 16};
    const int kcs[] = {64, 32, 16};  // K values per chunk (64 only for e4m3 slices)
    // explicit two-block splits of the bins first (they trade UMMA width for
    // drain overlap, which the cost model does not see), then the cost model's
    // best partition for each block count
    for (int bn : bns)
        for (int kc : kcs)
            for (int cut = 1; cut < cfg.J; ++cut) {
                PlanHints h;
                h.BN = bn;
                h.KC = kc;
                h.groups = 2;
                h.sizes[0] = cut;
                h.sizes[1] = cfg.J - cut;
                try_add(h);
            }
    for (int bn : bns)
        for (int kc : kcs)
            for (int g = 1; g <= kMaxGroups; ++g) {
                PlanHints h;
                h.BN = bn;
                h.KC = kc;
                h.groups = g;
                try_add(h);
            }
    // keep the candidates whose modelled UMMA cycles per output column are within
    // 35 % of the best, cheapest first (the untuned plan stays first)
    std::vector<double> score(plans.size());
    double best = 1e300;
    for (size_t i = 0; i < plans.size(); ++i) {
        score[i] = plans[i].model_cycles_per_kstep / plans[i].BN;
        best = std::min(best, score[i]);
    }
    std::vector<size_t> idx;
    for (size_t i = 1; i < plans.size(); ++i)
        if (score[i] <= 1.35 * best) idx.push_back(i);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return score[x] < score[y]; });
    std::vector<PlanHints> kept;
    if (!out.empty()) kept.push_back(out[0]);
    for (size_t i : idx)
        if (static_cast<int>(kept.size()) < max_n) kept.push_back(out[i]);
    return kept;
}

double knob_estimate(const KnobStats &k, int K, int b, int s, int crit, double tail) {
    return knob_estimate_set(k, K, b, s, s, crit, tail);
}

double knob_estimate_set(const KnobStats &k, int K, int b, int s, int J, int crit, double tail) {
    const double safety = 1.5;
    // first dropped pairs p + q = J (none for the full set), relative to the tails' 2^{-bs}
    const double nd = J < 2 * s - 1 ? static_cast<double>(pairs_in_bin(J, s)) : 0.0;
    const double wd = nd * std::ldexp(1.0, -b * (J - s));
    if (crit == KNOB_ELEMENTWISE) {
        // the largest of many entries' errors, about 4 of their standard deviations
        const double safety_max = 4.0;
        if (!(k.ia > 0.0) || !(k.ib > 0.0) || !(tail > 0.0)) return HUGE_VAL;
        const double Kd = static_cast<double>(K);
        const double r = Kd * wd * wd * k.ia * k.ib / 16.0 + (k.ia + k.ib) / 3.0;
        const double v = safety_max * std::ldexp(std::sqrt(Kd * r), -b * s) / tail + std::ldexp(1.0, -53);
        return std::isfinite(v) ? v : HUGE_VAL;
    }
    if (!(k.t > 0.0)) return HUGE_VAL;
    const double dropped = 0.25 * wd * std::sqrt(static_cast<double>(K) * k.sa * k.sb);
    const double tails = std::sqrt(k.sa * k.nb / 3.0) + std::sqrt(k.sb * k.na / 3.0);
    const double v = safety * std::ldexp((dropped + tails) / std::sqrt(k.t), -b * s) + std::ldexp(1.0, -53);
    return std::isfinite(v) ? v : HUGE_VAL;
}

double plan_time_model(const Plan &p, int M, int N, int K, int sms) {
    const double units = static_cast<double>(p.tiles_m) * p.tiles_n;
    const double waves = std::ceil(units / std::max(1, sms));
    const int k_per_umma = p.f8 ? 32 : 16;
    const double ksteps_per_chunk = static_cast<double>(p.KC / k_per_umma);
    const double gemm_s = waves * p.n_kc * ksteps_per_chunk * p.model_cycles_per_kstep / 2.0e9;
    const double split_bytes = 8.0 * (static_cast<double>(M) * K + static_cast<double>(K) * N) +
                               static_cast<double>(p.a_bytes + p.b_bytes);
    return 1e3 * (gemm_s + split_bytes / 6.5e12);
}

Schedule choose_schedule(const KnobStats &k, int M, int N, int K, const OzConfig &base, double bound, int s_min,
                         int s_max, int crit, double tail, bool any_set, int sms) {
    Schedule best;
    if (!any_set) {
        // the triangular set: the fewest slices that meet the bound
        double est = HUGE_VAL;
        const int s = choose_slices_stats(k, K, base.b, bound, s_min, s_max, &est, crit, tail);
        best.s = best.J = s;
        best.est = est;
        return best;
    }
    int first_ok = 0;
    for (int s = s_min; s <= s_max; ++s) {
        if (first_ok && s > first_ok + 3) break;  // a product with 4 more slices is not cheaper
        const int j_max = any_set ? std::min(2 * s - 1, 32) : s;
        // the estimate does not grow with J: no J meets the bound if the largest does not
        if (!(knob_estimate_set(k, K, base.b, s, std::max(s, j_max), crit, tail) <= bound)) continue;
        for (int J = s; J <= std::max(s, j_max); ++J) {
            const double est = knob_estimate_set(k, K, base.b, s, J, crit, tail);
            if (!(est <= bound)) continue;
            if (!first_ok) first_ok = s;
            OzConfig c = base;
            c.s = s;
            c.J = J;
            Plan p;
            std::string why;
            if (!make_plan(M, N, K, c, &p, &why)) break;  // a larger J needs at least as much
            const double ms = plan_time_model(p, M, N, K, sms);
            if (!best.s || ms < best.ms * (1.0 - 1e-9)) {
                best.s = s;
                best.J = J;
                best.est = est;
                best.ms = ms;
            }
            break;  // the smallest J meeting the bound for this s
        }
    }
    if (!best.s) {
        best.s = best.J = s_max;
        best.est = knob_estimate_set(k, K, base.b, s_max, s_max, crit, tail);
    }
    return best;
}

int choose_slices_stats(const KnobStats &k, int K, int b, double bound, int s_min, int s_max, double *estimate,
                        int crit, double tail) {
    int s = s_min;
    double est = HUGE_VAL;
    for (; s <= s_max; ++s) {
        est = knob_estimate(k, K, b, s, crit, tail);
        if (est <= bound) break;
    }
    if (s > s_max) s = s_max;
    if (estimate) *estimate = est;
    return s;
}

KnobStats knob_stats_host(const int32_t *er, const double *ssr, int M, const int32_t *ec, const double *ssc, int N,
                          const double *ca, const double *rb, int K) {
    int ea = 0, eb = 0;
    for (int i = 0; i < M; ++i) ea = std::max(ea, static_cast<int>(er[i]));
    for (int j = 0; j < N; ++j) eb = std::max(eb, static_cast<int>(ec[j]));
    long double sa = 0, na = 0, sb = 0, nb = 0, t = 0;
    for (int i = 0; i < M; ++i) {
        sa += std::ldexp(1.0L, 2 * (er[i] - ea));
        na += std::ldexp(static_cast<long double>(ssr[i]), -2 * (ea - 1022));
    }
    for (int j = 0; j < N; ++j) {
        sb += std::ldexp(1.0L, 2 * (ec[j] - eb));
        nb += std::ldexp(static_cast<long double>(ssc[j]), -2 * (eb - 1022));
    }
    if (ca && rb) {
        for (int k = 0; k < K; ++k)
            t += std::ldexp(static_cast<long double>(ca[k]), -2 * (ea - 1022)) *
                 std::ldexp(static_cast<long double>(rb[k]), -2 * (eb - 1022));
    } else {
        t = na * nb / K;
    }
    // the flattest row and column: max 1 / (|x|^2 4^{1022-E}) over the non-zero units
    long double ia = 0, ib = 0;
    for (int i = 0; i < M; ++i)
        if (ssr[i] > 0) ia = std::max(ia, 1.0L / std::ldexp(static_cast<long double>(ssr[i]), 2 * (1022 - er[i])));
    for (int j = 0; j < N; ++j)
        if (ssc[j] > 0) ib = std::max(ib, 1.0L / std::ldexp(static_cast<long double>(ssc[j]), 2 * (1022 - ec[j])));
    return KnobStats{static_cast<double>(sa), static_cast<double>(na), static_cast<double>(sb),
                     static_cast<double>(nb), static_cast<double>(t),  static_cast<double>(ia),
                     static_cast<double>(ib)};
}

}  // namespace ozgb
