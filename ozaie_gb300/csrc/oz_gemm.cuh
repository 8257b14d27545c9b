// oz_gemm.cuh -- stage (c) + (d): slice-pair GEMMs on tcgen05 with exact
// accumulation, fused with the FP64 reconstruction.
//
// Reference semantics (atlarge-research/ozAIE):
//   bins[p+q] += A_p . B_q over the pair set      src/aie_kernels/aie2p/mm_ozaki.cc:255-308
//   bins accumulate over all of K per C tile       whole_array_iron_ozaki.py:494-548
//   bin-weighted sum + exponent scale-back         src/aie_kernels/generic/ozaki_base.cc:143-340
//   int128 -> double reconstruction                include/oz_aie.h:92-150
//
// GB300 design (persistent CTAs, one per SM, each looping over 128 x BN tiles of
// C; 640 threads: a producer warp, 16 drain/epilogue warps and up to three
// MMA-issuing warps on three schedulers):
//   * Carrier: tcgen05.mma kind::f16 with bf16 slices (|v| <= 127 is exact in
//     bf16) and fp32 accumulators in TMEM.  (kind::i8 is not accepted by ptxas
//     for sm_103a.)  Slices of b <= 4 bits may instead be e4m3 (kind::f8f6f4,
//     template F8): a 64-deep e4m3 chunk has the byte layout of a 32-deep bf16
//     one, so only the instruction and its operand formats change.  Every
//     partial sum is an integer of magnitude <= 2^24 as
//     long as bin j accumulates at most KB_j K-values between drains,
//     pairs_in_bin(j) * KB_j * (2^b-1)^2 <= 2^24, so the fp32 accumulation is exact.
//   * TMEM holds one fp32 accumulator of BN columns per bin j (column j*BN), and
//     a second range for each double-buffered block where the columns allow it.
//     Bins are partitioned into up to 8 blocks of at most 256 columns.  Every
//     UMMA of a block spans the whole block: A slice p against the B slices
//     q = j - p of all bins j of the block, which are consecutive in shared
//     memory; q outside [0, s) reads zero slices padded below and above the
//     loaded ones.  On GB300 one M=128, K=16 UMMA occupies the tensor pipe for
//     N/2 cycles, and one issuing thread issues one about every 80-100 cycles,
//     so wide UMMAs from several issuers feed the pipe; the planner picks the
//     partition with a cost model fitted to this kernel.
//   * The UMMA runs of a K step (block, A slice) are dealt round-robin to the
//     issuing warps, which all accumulate (enable_input_d = 1): the drain warps
//     store zeros over every accumulator they read out, and TMEM starts zeroed.
//   * Each block is a drain group with its own period (its tightest bin).  In
//     each chunk the issuers first issue the blocks that drain after this chunk,
//     then the others, and last the blocks drained after the previous chunk
//     (after waiting for their drain): a drain overlaps the UMMAs of the other
//     blocks.  A double-buffered block switches ranges at each drain instead.
//   * Drain (warps 2..17): TMEM -> registers, fp32 -> int32 (exact), then one
//     32 x 32 -> 64-bit multiply-add by 2^rel into the 64-bit accumulator of the
//     bin's group (consecutive bins whose weights relative to the group's first
//     bin stay <= 2^30).  The W-word exact sum is assembled once per element in
//     the epilogue.  Integer ALU work competes with the MMA-issuing warps on their
//     schedulers, so the drain keeps it to two instructions per value.
//   * The last partial wave of a launch may be split along K (split_parts): the
//     parts add their 64-bit group sums into global scratch with atomics and
//     the part that completes a tile's count rounds and stores it.
//   * Epilogue: the exact accumulator q is rounded once to FP64 with the scale
//     2^{Er+Ec-2044-b(J+1)} (round-to-nearest, or the reference's truncating
//     decode, or written raw for parity dumps).
//   * Every mbarrier wait is bounded (globaltimer); on expiry the kernel records
//     an error code, waits for its own copies and MMAs, frees TMEM and returns.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "oz_internal.h"
#include "oz_ptx.cuh"

namespace ozgb {

// ------------------------------------------------------------ drain adds
// d = a * m + c with a 64-bit result: one multiply-add per drained value.
__device__ __forceinline__ long long mad_wide(int32_t a, int32_t m, long long c) {
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(m), "l"(c));
    return d;
}

// acc[i][A] += v[i] * 2^rel modulo 2^64 for NV fp32 values holding exact
// integers (|v| <= 2^24).  Exact-mode plans keep rel <= 30; the paired output
// of the reference (sums modulo 2^64) may need up to 63.
template <int NA, int A, int NV>
__device__ __forceinline__ void acc_add(long long (*acc)[NA], const uint32_t *v, int rel) {
    if (rel <= 30) {
        const int32_t m = 1 << rel;
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i][A] = mad_wide(__float2int_rz(__uint_as_float(v[i])), m, acc[i][A]);
    } else if (rel <= 36) {
        const int k = rel - 30;  // |v| 2^k < 2^31
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const uint32_t iv = static_cast<uint32_t>(__float2int_rz(__uint_as_float(v[i])));
            acc[i][A] = mad_wide(static_cast<int32_t>(iv << k), 1 << 30, acc[i][A]);
        }
    } else if (rel < 64) {
        const int k = rel - 32;  // only the high word changes (modulo 2^64)
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const uint32_t iv = static_cast<uint32_t>(__float2int_rz(__uint_as_float(v[i])));
            acc[i][A] += static_cast<long long>(static_cast<unsigned long long>(iv << k) << 32);
        }
    }
}

// The accumulator index is a template argument: a runtime index into acc would
// place the whole array in local memory.
template <int NA, int NV>
__device__ __forceinline__ void acc_add_group(long long (*acc)[NA], const uint32_t *v, int a, int rel) {
    switch (a) {
        case 0: acc_add<NA, 0, NV>(acc, v, rel); break;
        case 1: if constexpr (NA > 1) acc_add<NA, 1, NV>(acc, v, rel); break;
        case 2: if constexpr (NA > 2) acc_add<NA, 2, NV>(acc, v, rel); break;
        case 3: if constexpr (NA > 3) acc_add<NA, 3, NV>(acc, v, rel); break;
        default: break;
    }
}

// q += x * 2^sh for a signed 64-bit x, q two's complement in W words (epilogue).
template <int W>
__device__ __forceinline__ void q_add_i64(uint32_t (&q)[W], long long x, int sh) {
    const int k = sh >> 5, r = sh & 31;
    const uint32_t lo = static_cast<uint32_t>(x);
    const uint32_t hi = static_cast<uint32_t>(static_cast<unsigned long long>(x) >> 32);
    const uint32_t ext = static_cast<uint32_t>(x >> 63);
    const uint32_t p0 = lo << r, p1 = __funnelshift_l(lo, hi, r), p2 = __funnelshift_l(hi, ext, r);
    uint32_t carry = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        const int d = w - k;
        const uint32_t a = d < 0 ? 0u : d == 0 ? p0 : d == 1 ? p1 : d == 2 ? p2 : ext;
        const unsigned long long sum = static_cast<unsigned long long>(q[w]) + a + carry;
        q[w] = static_cast<uint32_t>(sum);
        carry = static_cast<uint32_t>(sum >> 32);
    }
}

// TMEM columns per load batch of a drain thread: the widest that divides its
// columns and leaves the accumulators (2 NA registers per column) room.
__host__ __device__ constexpr int drain_batch(int cols, int acc_regs) {
    return (cols % 16 == 0 && acc_regs + 16 <= 64)   ? 16
           : (cols % 12 == 0 && acc_regs + 12 <= 64) ? 12
           : (cols % 8 == 0 && acc_regs + 8 <= 64)   ? 8
                                                     : 4;
}

// ------------------------------------------------------------ q -> double
template <int W>
__device__ __forceinline__ uint32_t qword(const uint32_t (&m)[W], int i) {
    uint32_t r = 0;
#pragma unroll
    for (int t = 0; t < W; ++t) r = (t == i) ? m[t] : r;
    return r;
}
// floor(m / 2^sh) for sh >= 0 (low 64 bits), m << -sh for sh < 0.
template <int W>
__device__ __forceinline__ uint64_t qextract64(const uint32_t (&m)[W], int sh) {
    if (sh < 0) {
        const uint64_t lo = static_cast<uint64_t>(m[0]) | (W > 1 ? (static_cast<uint64_t>(m[1]) << 32) : 0ull);
        return (-sh >= 64) ? 0ull : (lo << (-sh));
    }
    const int wi = sh >> 5, bo = sh & 31;
    const uint32_t w0 = qword(m, wi), w1 = qword(m, wi + 1), w2 = qword(m, wi + 2);
    const uint32_t lo = __funnelshift_r(w0, w1, bo);
    const uint32_t hi = __funnelshift_r(w1, w2, bo);
    return (static_cast<uint64_t>(hi) << 32) | lo;
}
template <int W>
__device__ __forceinline__ int qbit(const uint32_t (&m)[W], int i) {
    if (i < 0) return 0;
    return static_cast<int>((qword(m, i >> 5) >> (i & 31)) & 1u);
}
template <int W>
__device__ __forceinline__ bool qany_below(const uint32_t (&m)[W], int i) {
    uint32_t acc = 0;
#pragma unroll
    for (int t = 0; t < W; ++t) {
        const int base = 32 * t;
        if (base + 32 <= i) acc |= m[t];
        else if (base < i) acc |= m[t] & ((1u << (i - base)) - 1u);
    }
    return acc != 0;
}

// value = q * 2^(escale - 2044 - bJ1), q two's complement in W words.
template <int W>
__device__ __forceinline__ double q_to_double(const uint32_t (&q)[W], int escale, int bJ1, int mode) {
    const bool neg = static_cast<int32_t>(q[W - 1]) < 0;
    uint32_t m[W];
    {
        uint32_t carry = 1;
#pragma unroll
        for (int t = 0; t < W; ++t) {
            const uint32_t x = neg ? ~q[t] : q[t];
            const uint32_t add = neg ? carry : 0u;
            const uint32_t s = x + add;
            carry = (neg && s < x) ? 1u : 0u;
            m[t] = s;
        }
    }
    int L = 0;
#pragma unroll
    for (int t = 0; t < W; ++t)
        if (m[t]) L = 32 * t + 32 - __clz(m[t]);
    if (L == 0) return 0.0;
    uint64_t bits;
    if (mode == OUT_RZ_REF) {
        // include/oz_aie.h:129-146: exponent = L - b(d+1) - 1, truncate to 53 bits,
        // lu = mant - 2^52 + sign + (exponent+1023)<<52 + (Er+Ec+2-2046)<<52 mod 2^64.
        const long long exponent = static_cast<long long>(L) - bJ1 - 1;
        uint64_t lu = qextract64(m, L - 53);
        lu -= 0x0010000000000000ull;
        lu += (neg ? 0x8000000000000000ull : 0ull) + (static_cast<uint64_t>(exponent + 1023) << 52) +
              (static_cast<uint64_t>(static_cast<long long>(escale) - 2044) << 52);
        bits = lu;
    } else {
        const int e2 = escale - 2044 - bJ1;
        const int biased = L - 1 + e2 + 1023;
        const int sh = (biased >= 1) ? L - 53 : L - 53 + (1 - biased);
        uint64_t mm = (sh > L) ? 0ull : qextract64(m, sh);
        const int rb = (sh - 1 >= L) ? 0 : qbit(m, sh - 1);
        const bool st = qany_below(m, sh - 1);
        if (rb && (st || (mm & 1ull))) mm++;
        if (biased >= 1) {
            if (biased >= 2047) {
                bits = 0x7FF0000000000000ull;
            } else {
                bits = (static_cast<uint64_t>(biased - 1) << 52) + mm;
                if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
            }
        } else {
            bits = mm;
        }
        if (neg) bits |= 0x8000000000000000ull;
    }
    return __longlong_as_double(static_cast<long long>(bits));
}

// The same rounding (OUT_RN) for q = a0 + a1 2^B with 0 <= B <= 63, the exact sum
// of at most two accumulator groups: one signed 128-bit integer, so the rounding
// needs no word selects.  Bit for bit the result of q_to_double.
__device__ __forceinline__ double acc2_to_double_rn(long long a0, long long a1, int B, int escale, int bJ1) {
    const __int128 S = static_cast<__int128>(a0) + (static_cast<__int128>(a1) << B);
    if (S == 0) return 0.0;
    const bool neg = S < 0;
    const unsigned __int128 m = neg ? static_cast<unsigned __int128>(-S) : static_cast<unsigned __int128>(S);
    const unsigned long long hi = static_cast<unsigned long long>(m >> 64), lo = static_cast<unsigned long long>(m);
    const int L = hi ? 128 - __clzll(static_cast<long long>(hi)) : 64 - __clzll(static_cast<long long>(lo));
    const int e2 = escale - 2044 - bJ1;
    const int biased = L - 1 + e2 + 1023;
    const int sh = (biased >= 1) ? L - 53 : L - 53 + (1 - biased);
    unsigned long long mm;
    if (sh < 0) mm = (-sh >= 64) ? 0ull : (lo << (-sh));  // L < 53: m is lo
    else mm = (sh > L) ? 0ull : static_cast<unsigned long long>(m >> sh);
    const int rpos = sh - 1;  // the rounding bit's position
    const int rb = (rpos < 0 || rpos >= L) ? 0 : static_cast<int>((m >> rpos) & 1u);
    bool st = false;          // any bit below the rounding bit
    if (rpos >= 128) st = true;  // m != 0
    else if (rpos > 0) st = (m & ((static_cast<unsigned __int128>(1) << rpos) - 1u)) != 0;
    if (rb && (st || (mm & 1ull))) mm++;
    uint64_t bits;
    if (biased >= 1) {
        if (biased >= 2047) {
            bits = 0x7FF0000000000000ull;
        } else {
            bits = (static_cast<uint64_t>(biased - 1) << 52) + mm;
            if (bits >= 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
        }
    } else {
        bits = mm;
    }
    if (neg) bits |= 0x8000000000000000ull;
    return __longlong_as_double(static_cast<long long>(bits));
}

// ------------------------------------------------------------ drain schedule
// Block g is drained after chunk c when (c + 1 + blk_off[g]) % blk_period[g] == 0,
// and every block after the last chunk.  The MMA issuer and the drain warps step
// identical copies of this schedule.
struct DrainSchedule {
    int r[kMaxGroups];
    __device__ __forceinline__ void init(const GemmArgs &g) {
#pragma unroll
        for (int i = 0; i < kMaxGroups; ++i) r[i] = (i < g.G) ? (1 + g.blk_off[i]) % g.blk_period[i] : 1;
    }
    // Mask of the blocks drained after the current chunk; advances to the next chunk.
    __device__ __forceinline__ uint32_t next(const GemmArgs &g, bool last) {
        uint32_t m = 0;
#pragma unroll
        for (int i = 0; i < kMaxGroups; ++i) {
            if (i < g.G) {
                if (r[i] == 0) m |= 1u << i;
                r[i] = (r[i] + 1 == g.blk_period[i]) ? 0 : r[i] + 1;
            }
        }
        return last ? ((1u << g.G) - 1u) : m;
    }
};

// ------------------------------------------------------------------ kernel
// The operands and output of one tile and its position.  Grouped rasterisation:
// 8 M-tiles share the same stream of B tiles.
struct TileRef {
    const uint8_t *a_src;
    const uint8_t *b_src;
    const int32_t *er;
    const int32_t *ec;
    double *c;
    long ldc;
    int M, N, n_kc, mt, nt;
    int c0, c1;  // chunks of K this work unit covers
    int split;   // index of the split tile (-1: the unit is a whole tile)
};

// Tile t of a problem whose tiles are rasterised in groups of 8 row tiles that
// share the same stream of B tiles.
OZ_HD inline void raster(int t, int tiles_m, int tiles_n, int *mt, int *nt) {
    const int GM = 8;
    const int per_group = GM * tiles_n;
    const int grp = t / per_group;
    const int first_m = grp * GM;
    const int gm = (tiles_m - first_m) < GM ? (tiles_m - first_m) : GM;
    const int rr = t - grp * per_group;
    *mt = first_m + rr % gm;
    *nt = rr / gm;
}

// Work unit u of a grouped launch: problem tile_prob[u], its tile u - tile0.
// Shared by the kernel and the host-side check of grouped launches.
OZ_HD inline void group_tile_ref(const GroupProblem *probs, const int *tile_prob, int u, uint32_t a_block_bytes,
                                 uint32_t b_block_bytes, TileRef *r) {
    const GroupProblem &P = probs[tile_prob[u]];
    r->split = -1;
    r->c0 = 0;
    r->c1 = P.n_kc;
    r->er = P.er;
    r->ec = P.ec;
    r->c = P.c;
    r->ldc = P.ldc;
    r->M = P.M;
    r->N = P.N;
    r->n_kc = P.n_kc;
    raster(u - P.tile0, P.tiles_m, P.tiles_n, &r->mt, &r->nt);
    r->a_src = P.a_tiles + static_cast<size_t>(r->mt) * P.n_kc * a_block_bytes;
    r->b_src = P.b_tiles + static_cast<size_t>(r->nt) * P.n_kc * b_block_bytes;
}

__device__ __forceinline__ void tile_ref(const GemmArgs &g, int u, TileRef *r) {
    if (g.probs) {
        group_tile_ref(g.probs, g.tile_prob, u, g.a_block_bytes, g.b_block_bytes, r);
        return;
    }
    int t = u, kpart = 0;
    r->split = -1;
    if (g.split_parts > 1 && u >= g.split_start) {
        const int v = u - g.split_start;
        r->split = v / g.split_parts;
        kpart = v - r->split * g.split_parts;
        t = g.split_start + r->split;
    }
    r->c0 = r->split < 0 ? 0 : (kpart * g.n_kc) / g.split_parts;
    r->c1 = r->split < 0 ? g.n_kc : ((kpart + 1) * g.n_kc) / g.split_parts;
    r->er = g.er;
    r->ec = g.ec;
    r->c = g.c;
    r->ldc = g.ldc;
    r->M = g.M;
    r->N = g.N;
    r->n_kc = g.n_kc;
    raster(t, g.tiles_m, g.tiles_n, &r->mt, &r->nt);
    r->a_src = reinterpret_cast<const uint8_t *>(g.a_tiles) + static_cast<size_t>(r->mt) * g.n_kc * g.a_block_bytes;
    r->b_src = reinterpret_cast<const uint8_t *>(g.b_tiles) + static_cast<size_t>(r->nt) * g.n_kc * g.b_block_bytes;
}

// Persistent: CTA b processes tiles b, b + gridDim.x, ...  The stage ring, the
// bin-block barriers and TMEM persist across tiles, so the producer prefetches
// the next tile's first chunks and the UMMAs of the next tile start as soon as
// each block's final drain of the previous tile has read it out, while the
// drain warps round and store the previous tile.
template <int BN, int W, int KC, bool F8>
__global__ void __launch_bounds__(kThreads, 1) oz_gemm_kernel(const __grid_constant__ GemmArgs g) {
    constexpr int PARTS = kEpiWarps / 4;          // drain warps sharing one TMEM lane quadrant
    constexpr int COLS = BN / PARTS;              // columns per drain thread
    constexpr int NA = W > 2 ? W - 1 : 1;         // 64-bit accumulator groups per column
    constexpr int DB = drain_batch(COLS, 2 * NA * COLS);
    static_assert(NA <= kMaxAcc, "accumulator groups");
    static_assert(COLS % 4 == 0 && COLS % DB == 0, "BN must split into 4-column parts");

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + static_cast<size_t>(g.stages) * g.stage_bytes);
    uint64_t *empty = full + g.stages;
    uint64_t *gfull = empty + g.stages;
    uint64_t *gempty = gfull + 2 * kMaxGroups;  // [block][buffer]: index 2 * blk + buf
    uint64_t *mma_done = gempty + 2 * kMaxGroups;
    uint64_t *split_bar = mma_done + 1;  // the drain warps' barrier around a split tile's count
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(split_bar + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    volatile int *vabort = abort_flag;
    // the drain warps' block table: TMEM column of bin lo of block g in buffer b
    // at [2 g + b], then lo at [2 kMaxGroups + g] and nb at [3 kMaxGroups + g]
    int *drn = abort_flag + 1;
    int *split_flag = drn + 4 * kMaxGroups;  // this CTA's part completed a split tile

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // zero B slices below and above the loaded ones (read by out-of-range pairs)
    {
        const uint32_t pad_hi_bytes = g.b_region_bytes - g.b_pad_lo_bytes - g.b_block_bytes;
        for (int st = 0; st < g.stages; ++st) {
            uint8_t *breg = smem + static_cast<size_t>(st) * g.stage_bytes + g.a_block_bytes;
            for (uint32_t i = threadIdx.x * 16; i < g.b_pad_lo_bytes; i += kThreads * 16)
                *reinterpret_cast<uint4 *>(breg + i) = make_uint4(0, 0, 0, 0);
            uint8_t *top = breg + g.b_pad_lo_bytes + g.b_block_bytes;
            for (uint32_t i = threadIdx.x * 16; i < pad_hi_bytes; i += kThreads * 16)
                *reinterpret_cast<uint4 *>(top + i) = make_uint4(0, 0, 0, 0);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    const int n_iss = g.n_iss < 1 ? 1 : (g.n_iss > kMaxIssuers ? kMaxIssuers : g.n_iss);  // MMA-issuing warps
    if (threadIdx.x == 0) {
        for (int i = 0; i < g.stages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], n_iss);
        }
        // a block's drain waits for every issuer that has runs in it: its runs are
        // consecutive run numbers, so min(runs, n_iss) issuers
        for (int i = 0; i < g.G; ++i) {
            const int runs = g.blk_p1[i] - g.blk_p0[i] + 1;
            const int contributors = runs < n_iss ? runs : n_iss;
            for (int b = 0; b < 2; ++b) {
                mbar_init(&gfull[2 * i + b], contributors);
                mbar_init(&gempty[2 * i + b], kEpiWarps);
            }
        }
        mbar_init(mma_done, n_iss);
        mbar_init(split_bar, kEpiWarps);
        for (int i = 0; i < g.G; ++i) {
            drn[2 * i] = g.blk_lo[i] * BN;
            drn[2 * i + 1] = ((g.dbl_mask >> i) & 1u) ? g.blk_col1[i] : g.blk_lo[i] * BN;
            drn[2 * kMaxGroups + i] = g.blk_lo[i];
            drn[3 * kMaxGroups + i] = g.blk_nb[i];
        }
        *abort_flag = (*reinterpret_cast<volatile int *>(g.err) != 0) ? 1 : 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, g.tmem_cols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint64_t TO = g.timeout_ns;
    // Every UMMA accumulates, so TMEM starts zeroed (and each drain leaves what it
    // read zeroed): drain warp (quadrant qd, part) clears its quarter of the columns.
    if (warp >= 2 && warp < 2 + kEpiWarps) {
        const uint32_t quarter = g.tmem_cols >> 2;
        const uint32_t base = tmem + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + ((warp - 2) >> 2) * quarter;
        for (uint32_t col = 0; col < quarter; col += 8) tmem_st8_zero(base + col);
        tmem_st_wait();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp == 0) {
        // ------------------------------------------------------ producer
        if (lane == 0) {
            long long issued = 0;  // stage uses by this CTA over all of its tiles
            int st = 0;
            bool ok = true;
            // waits until stage st may be refilled: use r (>= 1) of a stage waits for
            // the (r-1)-th release of that stage
            auto acquire = [&]() -> bool {
                const long long r = issued / g.stages;
                const bool got = (r == 0) || mbar_wait(&empty[st], static_cast<uint32_t>((r - 1) & 1), vabort, TO);
                if (!got && !*vabort) {
                    atomicCAS(g.err, 0, DEVERR_TIMEOUT_PRODUCER);
                    *vabort = 1;
                }
                return got;
            };
            for (int t = g.tile_begin + static_cast<int>(blockIdx.x); ok && t < g.total_tiles; t += gridDim.x) {
                TileRef tr;
                tile_ref(g, t, &tr);
                for (int c = tr.c0; c < tr.c1; ++c) {
                    if (*vabort || !acquire()) {
                        ok = false;
                        break;
                    }
                    uint8_t *dst = smem + static_cast<size_t>(st) * g.stage_bytes;
                    mbar_arrive_expect_tx(&full[st], g.a_block_bytes + g.b_block_bytes);
                    bulk_g2s(dst, tr.a_src + static_cast<size_t>(c) * g.a_block_bytes, g.a_block_bytes, &full[st]);
                    bulk_g2s(dst + g.a_block_bytes + g.b_pad_lo_bytes,
                             tr.b_src + static_cast<size_t>(c) * g.b_block_bytes, g.b_block_bytes, &full[st]);
                    ++issued;
                    if (++st == g.stages) st = 0;
                }
            }
            // every copy issued must land before the CTA may exit
            const int zero = 0;
            const long long first = issued - g.stages;
            for (long long c = (first > 0 ? first : 0); c < issued; ++c)
                mbar_wait(&full[c % g.stages], static_cast<uint32_t>((c / g.stages) & 1), &zero, TO);
        }
    } else if (warp == 1 || warp >= kIssuer2Warp) {
        // ---------------------------------------------------- MMA issuers
        // Up to three issuing warps (on different SM sub-partitions), each run warp-wide
        // with lane 0 issuing and committing.  The UMMA runs of a K step (block g,
        // A slice p: ksteps UMMAs) are numbered block by block and dealt round-robin:
        // issuer iss takes the runs r with r % n_iss == iss.  Every UMMA accumulates
        // (the drain warps leave the accumulators they read out zeroed), so the
        // issuers of one block need no ordering among themselves.
        const int iss = warp == 1 ? 0 : warp - kIssuer2Warp + 1;
        if (iss < n_iss) {
            constexpr uint32_t a_step = (BM * KC * 2) >> 4;  // descriptor units (16 B)
            constexpr uint32_t b_step = (BN * KC * 2) >> 4;
            constexpr uint32_t sbo = KC * 16;
            constexpr int ksteps = KC >> 4;
            const uint32_t a0 = smem_u32(smem);
            const uint64_t ad0 = smem_desc(a0, 128, sbo);
            const uint64_t bd0 = smem_desc(a0 + g.a_block_bytes + g.b_pad_lo_bytes, 128, sbo);
            const uint32_t idesc_base = (F8 ? idesc_e4m3_f32(BM, 16) : idesc_bf16_f32(BM, 16)) & ~(0x3Fu << 17);
            // block table in the lanes (lane i: block i): bins, A slices, second buffer,
            // and this issuer's first A slice in the block (> p1: no runs there)
            int t_lo = 0, t_nb = 0, t_p0 = 0, t_p1 = -1, t_c1 = 0;
#pragma unroll
            for (int i = 0; i < kMaxGroups; ++i)
                if (lane == i && i < g.G) {
                    t_lo = g.blk_lo[i];
                    t_nb = g.blk_nb[i];
                    t_p0 = g.blk_p0[i];
                    t_p1 = g.blk_p1[i];
                    t_c1 = g.blk_col1[i];
                }
            const int runs = t_p1 - t_p0 + 1;
            int incl = runs;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            const int rb = incl - runs;  // runs of the blocks before this one
            const int t_pf = t_p0 + ((iss - rb % n_iss) % n_iss + n_iss) % n_iss;
            const uint32_t mine = __ballot_sync(0xffffffffu, lane < g.G && t_pf <= t_p1);
            const uint32_t dbl = g.dbl_mask & mine;  // double-buffered: UMMAs go on during their drains
            uint32_t ephase = 0;  // parity of the gempty waits, bit 2 blk + buf
            uint32_t pend = 0;    // drains committed and not yet waited for, bit 2 blk + buf
            uint32_t bufm = 0;    // accumulator buffer each block writes now
            uint32_t prev = 0;    // single-buffered blocks drained after the previous chunk
            int st = 0;
            uint32_t fparity = 0;
            bool ok = true;
            for (int t = g.tile_begin + static_cast<int>(blockIdx.x); ok && t < g.total_tiles; t += gridDim.x) {
                TileRef tr;
                tile_ref(g, t, &tr);
                DrainSchedule ds;
                ds.init(g);
                for (int c = tr.c0; c < tr.c1; ++c) {
                    const uint32_t cur = ds.next(g, c == tr.c1 - 1);
                    int got = 1;
                    if (lane == 0) got = mbar_wait(&full[st], fparity, vabort, TO) ? 1 : 0;
                    if (!__shfl_sync(0xffffffffu, got, 0)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t stage_off = (static_cast<uint64_t>(st) * g.stage_bytes) >> 4;
                    // issue order: blocks drained after this chunk, then the rest, then the
                    // blocks whose drain (after the previous chunk) must finish first
                    const uint32_t order[3] = {cur & mine & ~prev, mine & ~cur & ~prev, prev};
                    for (int cls = 0; ok && cls < 3; ++cls) {
                        uint32_t m = order[cls];
                        while (m) {
                            const int blk = __ffs(m) - 1;
                            const uint32_t bit = 1u << blk;
                            m &= m - 1;
                            const int lo = __shfl_sync(0xffffffffu, t_lo, blk);
                            const int nb = __shfl_sync(0xffffffffu, t_nb, blk);
                            const int p1 = __shfl_sync(0xffffffffu, t_p1, blk);
                            const int pf = __shfl_sync(0xffffffffu, t_pf, blk);
                            const int c1 = __shfl_sync(0xffffffffu, t_c1, blk);
                            const int bb = static_cast<int>((bufm >> blk) & 1u);
                            const int ix = 2 * blk + bb;
                            if ((pend >> ix) & 1u) {
                                // the buffer's previous drain must have read it out
                                int gote = 1;
                                if (lane == 0) gote = mbar_wait(&gempty[ix], (ephase >> ix) & 1u, vabort, TO) ? 1 : 0;
                                if (!__shfl_sync(0xffffffffu, gote, 0)) {
                                    ok = false;
                                    break;
                                }
                                ephase ^= 1u << ix;
                                pend &= ~(1u << ix);
                                tc_fence_after();
                            }
                            const uint32_t d_tmem = tmem + static_cast<uint32_t>(bb ? c1 : lo * BN);
                            const uint32_t idesc = idesc_base | (static_cast<uint32_t>((nb * BN) >> 3) << 17);
                            for (int p = pf; p <= p1; p += n_iss) {
                                // A slice p against B slices q = j - p of the block's bins j
                                const uint64_t ad = ad0 + stage_off + static_cast<uint64_t>(p) * a_step;
                                const uint64_t bd =
                                    bd0 + stage_off + static_cast<uint64_t>(static_cast<int64_t>(lo - p) * b_step);
                                if (lane == 0) {
#pragma unroll
                                    for (int kk = 0; kk < ksteps; ++kk) {
                                        // one UMMA covers 32 bytes of K per row: 16 bf16 or 32 e4m3 values
                                        if constexpr (F8)
                                            umma_e4m3(d_tmem, ad + static_cast<uint64_t>(kk * 16),
                                                      bd + static_cast<uint64_t>(kk * 16), idesc, 1u);
                                        else
                                            umma_bf16(d_tmem, ad + static_cast<uint64_t>(kk * 16),
                                                      bd + static_cast<uint64_t>(kk * 16), idesc, 1u);
                                    }
                                }
                            }
                            if (cur & bit) {
                                if (lane == 0) umma_commit(&gfull[ix]);
                                pend |= 1u << ix;
                                if (dbl & bit) bufm ^= bit;
                            }
                        }
                    }
                    if (!ok) break;
                    if (lane == 0) umma_commit(&empty[st]);
                    if (++st == g.stages) {
                        st = 0;
                        fparity ^= 1u;
                    }
                    prev = cur & mine & ~dbl;
                }
            }
            if (!ok && lane == 0 && !*vabort) {
                atomicCAS(g.err, 0, DEVERR_TIMEOUT_MMA);
                *vabort = 1;
            }
            // all MMAs issued by this warp complete before TMEM is released
            if (lane == 0) {
                umma_commit(mma_done);
                const int zero = 0;
                mbar_wait(mma_done, 0, &zero, TO);
            }
        }
        __syncwarp();
    } else {
        // ------------------------------------------ drain + epilogue warps
        const int ew = warp - 2;
        const int qd = warp & 3;  // TMEM lane quadrant accessible to this warp
        const int part = ew >> 2;  // which COLS-wide column slice of the tile
        const uint32_t trow = tmem + (static_cast<uint32_t>(32 * qd) << 16) + static_cast<uint32_t>(part * COLS);

        long long acc[COLS][NA];
        uint32_t fphase = 0;  // parity of the gfull waits, bit 2 blk + buf
        uint32_t dbuf = 0;    // accumulator buffer each block's next drain reads
        uint32_t prev = 0;
        bool ok = true;
        // barrier of the 16 drain warps (one arrival per warp), with the bounded wait
        // of every other barrier: a warp that gave up cannot leave the others waiting
        uint32_t sphase = 0;
        auto drain_bar = [&]() -> bool {
            __syncwarp();
            if (lane == 0) mbar_arrive(split_bar);
            const bool got = mbar_wait(split_bar, sphase, vabort, TO);
            sphase ^= 1u;
            return got;
        };
        for (int t = g.tile_begin + static_cast<int>(blockIdx.x); ok && t < g.total_tiles; t += gridDim.x) {
            TileRef tr;
            tile_ref(g, t, &tr);
#pragma unroll
            for (int i = 0; i < COLS; ++i)
#pragma unroll
                for (int a = 0; a < NA; ++a) acc[i][a] = 0;

            DrainSchedule ds;
            ds.init(g);
            for (int c = tr.c0; ok && c < tr.c1; ++c) {
                const bool last = (c == tr.c1 - 1);
                const uint32_t cur = ds.next(g, last);
                for (int pass = 0; ok && pass < 2; ++pass) {
                    uint32_t m = pass == 0 ? (cur & ~prev) : (cur & prev);
                    while (m) {
                        const int blk = __ffs(m) - 1;
                        m &= m - 1;
                        const int bb = static_cast<int>((dbuf >> blk) & 1u);
                        const int ix = 2 * blk + bb;
                        const bool gotg = mbar_wait(&gfull[ix], (fphase >> ix) & 1u, vabort, TO);
                        if (!gotg) {
                            ok = false;
                            break;
                        }
                        fphase ^= 1u << ix;
                        tc_fence_after();
                        const int lo = drn[2 * kMaxGroups + blk];
                        const int hi = lo + drn[3 * kMaxGroups + blk] - 1;
                        // bin j of the buffer read is at column drn[ix] + (j - lo) BN
                        const uint32_t bbase = trow + static_cast<uint32_t>(drn[ix] - lo * BN);
                        for (int j = lo; j <= hi; ++j) {
                            // accumulator group of bin j and its weight within the group
                            const int t = g.J - 1 - j;
                            int a = 0, t0 = 0;
#pragma unroll
                            for (int x = 1; x < NA; ++x)
                                if (x < g.n_acc && t >= g.acc_t0[x]) {
                                    a = x;
                                    t0 = g.acc_t0[x];
                                }
                            const int rel = g.b * (t - t0);
#pragma unroll
                            for (int cb = 0; cb < COLS / DB; ++cb) {
                                uint32_t v[DB];
                                const uint32_t taddr = bbase + static_cast<uint32_t>(j * BN + cb * DB);
                                tmem_ld_cols<DB>(taddr, v);
                                tmem_ld_wait();
                                tmem_zero_cols<DB>(taddr);  // the next UMMAs accumulate onto zero
#pragma unroll
                                for (int i = 0; i < DB; ++i) reg_fence(v[i]);
                                acc_add_group<NA, DB>(acc + cb * DB, v, a, rel);
                            }
                        }
                        // the buffer is zeroed and free for the block's UMMAs again
                        tmem_st_wait();
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&gempty[ix]);
                        if ((g.dbl_mask >> blk) & 1u) dbuf ^= 1u << blk;
                    }
                }
                prev = cur & ~g.dbl_mask;
            }
            if (!ok) break;

            if (tr.split >= 0) {
                // a part of a split tile: add the exact group sums into the tile's
                // scratch (integer adds, exact in any order); the part that completes
                // the tile's count reads the totals and runs the epilogue
                unsigned long long *sa = g.split_acc + static_cast<size_t>(tr.split) * (NA * BN * BM);
                const int rl = 32 * qd + lane;
#pragma unroll
                for (int i = 0; i < COLS; ++i)
#pragma unroll
                    for (int a = 0; a < NA; ++a)
                        if (a < g.n_acc)
                            atomicAdd(sa + (static_cast<size_t>(a) * BN + part * COLS + i) * BM + rl,
                                      static_cast<unsigned long long>(acc[i][a]));
                __threadfence();
                if (!drain_bar()) {
                    ok = false;
                    break;
                }
                if (ew == 0 && lane == 0)
                    *split_flag = (atomicAdd(g.split_cnt + tr.split, 1) == g.split_parts - 1) ? 1 : 0;
                if (!drain_bar()) {
                    ok = false;
                    break;
                }
                if (!*reinterpret_cast<volatile int *>(split_flag)) continue;
                __threadfence();
                // the totals, leaving the scratch zero for the next launch
#pragma unroll
                for (int i = 0; i < COLS; ++i)
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                        acc[i][a] = 0;
                        if (a < g.n_acc) {
                            unsigned long long *ptr = sa + (static_cast<size_t>(a) * BN + part * COLS + i) * BM + rl;
                            acc[i][a] = static_cast<long long>(__ldcg(ptr));
                            __stcg(ptr, 0ull);
                        }
                    }
                if (ew == 0 && lane == 0) g.split_cnt[tr.split] = 0;
            }

            // --------------------------------------------------- epilogue
            const int row = tr.mt * BM + 32 * qd + lane;
            const int col0 = tr.nt * BN + part * COLS;
            if (row < tr.M) {
                // the scale exponents first, as independent loads, so that their
                // latency is paid once rather than once per column
                const int er = __ldg(tr.er + row);
                int es[COLS];
#pragma unroll
                for (int i = 0; i < COLS; ++i) es[i] = er + (col0 + i < tr.N ? __ldg(tr.ec + col0 + i) : 0);
                const int bJ1 = g.b * (g.J + 1);
                // the exact sum of column i: sum_a acc[i][a] 2^(b acc_t0[a]) in W words
                auto exact_q = [&](int i, uint32_t (&q)[W]) {
#pragma unroll
                    for (int w = 0; w < W; ++w) q[w] = 0;
#pragma unroll
                    for (int x = 0; x < NA; ++x)
                        if (x < g.n_acc) q_add_i64<W>(q, acc[i][x], g.b * g.acc_t0[x]);
                };
                if (g.out_mode == OUT_PAIRS) {
                    // the reference's device output: lo, then hi with bits 51..62 = Er + Ec
#pragma unroll
                    for (int i = 0; i < COLS; ++i) {
                        const int col = col0 + i;
                        if (col < tr.N) {
                            long long *dst =
                                reinterpret_cast<long long *>(g.raw) + (static_cast<size_t>(row) * tr.N + col) * 2;
                            const unsigned long long lo = static_cast<unsigned long long>(acc[i][0]);
                            unsigned long long hi = 0;
                            if constexpr (NA > 1) hi = g.n_acc > 1 ? static_cast<unsigned long long>(acc[i][1]) : 0ull;
                            const unsigned long long scale =
                                static_cast<unsigned long long>(static_cast<uint32_t>(es[i]));
                            hi = (hi & 0x8007FFFFFFFFFFFFull) | ((scale & 0xFFFull) << 51);
                            dst[0] = static_cast<long long>(lo);
                            dst[1] = static_cast<long long>(hi);
                        }
                    }
                } else if (g.out_mode == OUT_RAW) {
#pragma unroll
                    for (int i = 0; i < COLS; ++i) {
                        const int col = col0 + i;
                        if (col < tr.N) {
                            uint32_t q[W];
                            exact_q(i, q);
                            int32_t *dst = g.raw + (static_cast<size_t>(row) * tr.N + col) * 4;
                            const uint32_t ext = static_cast<uint32_t>(static_cast<int32_t>(q[W - 1]) >> 31);
#pragma unroll
                            for (int w = 0; w < 4; ++w) dst[w] = static_cast<int32_t>(w < W ? q[w] : ext);
                        }
                    }
                } else {
                    double *crow = tr.c + static_cast<size_t>(row) * tr.ldc;
                    const bool plain = g.alpha == 1.0 && g.beta == 0.0;
                    // pairs of columns as one 16-byte store where aligned (fewer, larger
                    // writes, which matters most when C is host memory)
                    const bool vec = (reinterpret_cast<uintptr_t>(crow + col0) & 15) == 0;
                    // at most two accumulator groups, the second at most 63 bits up: the
                    // 128-bit rounding path
                    const int B1 = g.n_acc > 1 ? g.b * g.acc_t0[1] : 0;
                    const bool two_groups = g.out_mode == OUT_RN && g.n_acc <= 2 && B1 <= 63;
#pragma unroll
                    for (int i = 0; i < COLS; i += 2) {
                        double v[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int col = col0 + i + u;
                            v[u] = 0.0;
                            if (col < tr.N) {
                                if (two_groups) {
                                    long long a1 = 0;
                                    if constexpr (NA > 1) a1 = g.n_acc > 1 ? acc[i + u][1] : 0ll;
                                    v[u] = acc2_to_double_rn(acc[i + u][0], a1, B1, es[i + u], bJ1);
                                } else {
                                    uint32_t q[W];
                                    exact_q(i + u, q);
                                    v[u] = q_to_double<W>(q, es[i + u], bJ1, g.out_mode);
                                }
                                // BLAS semantics: C is not read when beta == 0
                                if (!plain)
                                    v[u] = g.beta == 0.0 ? g.alpha * v[u] : fma(g.beta, crow[col], g.alpha * v[u]);
                            }
                        }
                        const int col = col0 + i;
                        if (vec && col + 1 < tr.N) {
                            *reinterpret_cast<double2 *>(crow + col) = make_double2(v[0], v[1]);
                        } else {
                            if (col < tr.N) crow[col] = v[0];
                            if (col + 1 < tr.N) crow[col + 1] = v[1];
                        }
                    }
                }
            }
        }
        if (!ok && !*vabort) {
            atomicCAS(g.err, 0, DEVERR_TIMEOUT_EPI);
            *vabort = 1;
        }
    }

    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, g.tmem_cols);
    }
}

// Number of SMs of the current device (one persistent CTA each).
inline int device_sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cached[dev] = n;
    }
    return cached[dev];
}

// F8: e4m3 slices (kind::f8f6f4); KC is then the bf16-equivalent chunk (bytes / 2
// per row and slice), i.e. half the K values the chunk holds.
template <int BN, int W, int KC, bool F8 = false>
void launch_gemm_variant(const GemmArgs &args, int tiles, size_t smem, void *stream) {
    auto kern = oz_gemm_kernel<BN, W, KC, F8>;
    // the shared-memory limit is raised once per device to the opt-in maximum (a
    // per-launch attribute call costs more than the launch itself; every caller
    // sets the same value, so two host threads that both make the first call only
    // repeat the same attribute call)
    static std::atomic<bool> raised[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !raised[dev].load(std::memory_order_acquire)) {
        int opt = 0;
        cudaDeviceGetAttribute(&opt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             opt > static_cast<int>(smem) ? opt : static_cast<int>(smem));
        if (dev >= 0 && dev < 64) raised[dev].store(true, std::memory_order_release);
    }
    const int range = args.total_tiles - args.tile_begin;
    const int grid = range < device_sm_count() ? range : device_sm_count();
    (void)tiles;
    kern<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(args);
}

}  // namespace ozgb
