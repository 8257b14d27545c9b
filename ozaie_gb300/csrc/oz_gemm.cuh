// oz_gemm.cuh -- stage (c) + (d): slice-pair GEMMs on tcgen05 with exact
// accumulation, fused with the FP64 reconstruction.
//
// Reference semantics (atlarge-research/ozAIE):
//   bins[p+q] += A_p . B_q over the pair set      src/aie_kernels/aie2p/mm_ozaki.cc:255-308
//   bins accumulate over all of K per C tile       whole_array_iron_ozaki.py:494-548
//   bin-weighted sum + exponent scale-back         src/aie_kernels/generic/ozaki_base.cc:143-340
//   int128 -> double reconstruction                include/oz_aie.h:92-150
//
// GB300 design (one CTA per 128 x BN tile of C, 320 threads):
//   * Carrier: tcgen05.mma kind::f16 with bf16 slices (|v| <= 127 is exact in
//     bf16) and fp32 accumulators in TMEM.  (kind::i8 is not accepted by ptxas
//     for sm_103a.)  Every partial sum is an integer of magnitude <= 2^24 as
//     long as a bin accumulates at most KB = KBc*KC K-values between drains,
//     pairs_in_bin * KB * (2^b-1)^2 <= 2^24, so the fp32 accumulation is exact.
//   * TMEM holds one fp32 accumulator of BN columns per bin j (column j*BN).
//     All pairs (p, q) of a bin group that share A_p are one MMA: the B slices
//     q = j-p for consecutive bins j are consecutive in shared memory and the
//     bins are consecutive in TMEM, so A_p is read once per group, not per pair.
//   * Bins are split into G contiguous groups; group g is drained after chunks
//     c with (c+1) % KBc == g.  The MMA issuer walks the groups of a chunk in
//     the rotation (c+1+t) % KBc, so the group that drains after this chunk is
//     issued first and the group drained after the previous chunk is issued
//     last: the drain of one group overlaps the MMAs of all the others.
//   * Drain (warps 2..9): TMEM -> registers, fp32 -> int32 (exact), shifted by
//     b(J-1-j) and added into a W-word two's complement accumulator per
//     element; the columns are then zeroed for the next period.
//   * Epilogue: the exact accumulator q is rounded once to FP64 with the scale
//     2^{Er+Ec-2044-b(J+1)} (round-to-nearest, or the reference's truncating
//     decode, or written raw for parity dumps).
//   * Every mbarrier wait is bounded (globaltimer); on expiry the kernel records
//     an error code, waits for its own copies and MMAs, frees TMEM and returns.
#pragma once
#include <cuda_runtime.h>

#include "oz_internal.h"
#include "oz_ptx.cuh"

namespace ozgb {

// ------------------------------------------------------------------ q adds
// q += lo * 2^(32*K0) + hi * 2^(32*(K0+1)) + ext * (2^(32*(K0+2)) + ...), one carry chain.
template <int W, int K0>
struct QAdd;

#define OZ_QADD_BODY_1(a) "add.u32 %" #a ", %" #a ", %W0;\n\t"

template <>
struct QAdd<2, 0> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t) {
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(q[0]), "+r"(q[1]) : "r"(lo), "r"(hi));
    }
};
template <>
struct QAdd<2, 1> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t, uint32_t) { q[1] += lo; }
};
template <>
struct QAdd<3, 0> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
            : "+r"(q[0]), "+r"(q[1]), "+r"(q[2])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<3, 1> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t) {
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(q[1]), "+r"(q[2]) : "r"(lo), "r"(hi));
    }
};
template <>
struct QAdd<3, 2> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t, uint32_t) { q[2] += lo; }
};
template <>
struct QAdd<4, 0> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.cc.u32 %2, %2, %6;\n\taddc.u32 %3, %3, %6;"
            : "+r"(q[0]), "+r"(q[1]), "+r"(q[2]), "+r"(q[3])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<4, 1> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
            : "+r"(q[1]), "+r"(q[2]), "+r"(q[3])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<4, 2> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t) {
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(q[2]), "+r"(q[3]) : "r"(lo), "r"(hi));
    }
};
template <>
struct QAdd<4, 3> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t, uint32_t) { q[3] += lo; }
};
template <>
struct QAdd<5, 0> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %5;\n\taddc.cc.u32 %1, %1, %6;\n\taddc.cc.u32 %2, %2, %7;\n\t"
            "addc.cc.u32 %3, %3, %7;\n\taddc.u32 %4, %4, %7;"
            : "+r"(q[0]), "+r"(q[1]), "+r"(q[2]), "+r"(q[3]), "+r"(q[4])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<5, 1> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.cc.u32 %2, %2, %6;\n\taddc.u32 %3, %3, %6;"
            : "+r"(q[1]), "+r"(q[2]), "+r"(q[3]), "+r"(q[4])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<5, 2> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t ext) {
        asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
            : "+r"(q[2]), "+r"(q[3]), "+r"(q[4])
            : "r"(lo), "r"(hi), "r"(ext));
    }
};
template <>
struct QAdd<5, 3> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t hi, uint32_t) {
        asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(q[3]), "+r"(q[4]) : "r"(lo), "r"(hi));
    }
};
template <>
struct QAdd<5, 4> {
    __device__ __forceinline__ static void run(uint32_t *q, uint32_t lo, uint32_t, uint32_t) { q[4] += lo; }
};

// Adds the n values v[] (fp32 holding exact integers) shifted left by 32*K0 + r
// into the accumulators q[0..n).
template <int W, int K0, int NV>
__device__ __forceinline__ void q_add_block(uint32_t (*q)[W], const uint32_t *v, int r) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        const int32_t iv = __float2int_rz(__uint_as_float(v[i]));
        const uint32_t ext = static_cast<uint32_t>(iv >> 31);
        const uint32_t lo = static_cast<uint32_t>(iv) << r;
        const uint32_t hi = __funnelshift_l(static_cast<uint32_t>(iv), ext, r);
        QAdd<W, K0>::run(q[i], lo, hi, ext);
    }
}

template <int W, int NV>
__device__ __forceinline__ void q_add_shifted(uint32_t (*q)[W], const uint32_t *v, int sh) {
    const int k = sh >> 5, r = sh & 31;
    switch (k) {
        case 0: q_add_block<W, 0, NV>(q, v, r); break;
        case 1: if constexpr (W > 1) q_add_block<W, 1, NV>(q, v, r); break;
        case 2: if constexpr (W > 2) q_add_block<W, 2, NV>(q, v, r); break;
        case 3: if constexpr (W > 3) q_add_block<W, 3, NV>(q, v, r); break;
        case 4: if constexpr (W > 4) q_add_block<W, 4, NV>(q, v, r); break;
        default: break;
    }
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

// ------------------------------------------------------------------ kernel
template <int BN, int W>
__global__ void __launch_bounds__(kThreads, 1) oz_gemm_kernel(const __grid_constant__ GemmArgs g) {
    constexpr int HALF = BN / 2;        // columns per drain thread
    constexpr int NLD = HALF / 8;       // 8-column TMEM loads per bin
    constexpr int MAXB = 256 / BN;      // bins per MMA (N <= 256)
    constexpr int DB = (HALF % 16 == 0) ? 16 : 8;  // columns per drain batch
    static_assert(HALF % 8 == 0, "BN must be a multiple of 16");

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + static_cast<size_t>(g.stages) * g.stage_bytes);
    uint64_t *empty = full + g.stages;
    uint64_t *gfull = empty + g.stages;
    uint64_t *gempty = gfull + g.G;
    uint64_t *tmem_ready = gempty + g.G;
    uint64_t *mma_done = tmem_ready + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);
    volatile int *vabort = abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // grouped rasterisation: 8 M-tiles share the same stream of B tiles
    int mt, nt;
    {
        const int GM = 8;
        const int t = blockIdx.x;
        const int per_group = GM * g.tiles_n;
        const int grp = t / per_group;
        const int first_m = grp * GM;
        const int gm = min(GM, g.tiles_m - first_m);
        const int r = t - grp * per_group;
        mt = first_m + r % gm;
        nt = r / gm;
    }

    if (threadIdx.x == 0) {
        for (int i = 0; i < g.stages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < g.G; ++i) {
            mbar_init(&gfull[i], 1);
            mbar_init(&gempty[i], kEpiWarps);
        }
        mbar_init(tmem_ready, kEpiWarps);
        mbar_init(mma_done, 1);
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

    if (warp == 0) {
        // ------------------------------------------------------ producer
        if (lane == 0) {
            const uint8_t *a_src = reinterpret_cast<const uint8_t *>(g.a_tiles) +
                                   static_cast<size_t>(mt) * g.n_kc * g.a_block_bytes;
            const uint8_t *b_src = reinterpret_cast<const uint8_t *>(g.b_tiles) +
                                   static_cast<size_t>(nt) * g.n_kc * g.b_block_bytes;
            int issued = 0;
            for (int c = 0; c < g.n_kc; ++c) {
                if (*vabort) break;
                const int st = c % g.stages, round = c / g.stages;
                if (round > 0 && !mbar_wait(&empty[st], (round - 1) & 1, vabort, TO)) {
                    if (!*vabort) {
                        atomicCAS(g.err, 0, DEVERR_TIMEOUT_PRODUCER);
                        *vabort = 1;
                    }
                    break;
                }
                uint8_t *dst = smem + static_cast<size_t>(st) * g.stage_bytes;
                mbar_arrive_expect_tx(&full[st], g.a_block_bytes + g.b_block_bytes);
                bulk_g2s(dst, a_src + static_cast<size_t>(c) * g.a_block_bytes, g.a_block_bytes, &full[st]);
                bulk_g2s(dst + g.a_block_bytes, b_src + static_cast<size_t>(c) * g.b_block_bytes, g.b_block_bytes,
                         &full[st]);
                ++issued;
            }
            // every copy issued must land before the CTA may exit
            const int zero = 0;
            for (int c = (issued > g.stages ? issued - g.stages : 0); c < issued; ++c)
                mbar_wait(&full[c % g.stages], (c / g.stages) & 1, &zero, TO);
        }
    } else if (warp == 1) {
        // ---------------------------------------------------- MMA issuer
        if (lane == 0) {
            bool ok = mbar_wait(tmem_ready, 0, vabort, TO);
            tc_fence_after();
            uint64_t ephase = 0;  // per-group parity of gempty waits
            const uint32_t idesc_base = idesc_bf16_f32(BM, 16) & ~(0x3Fu << 17);
            const uint32_t a_slice_bytes = BM * g.KC * 2;
            const uint32_t b_slice_bytes = BN * g.KC * 2;
            const uint32_t sbo = g.KC * 16;
            for (int c = 0; ok && c < g.n_kc; ++c) {
                const int st = c % g.stages, round = c / g.stages;
                if (!mbar_wait(&full[st], round & 1, vabort, TO)) { ok = false; break; }
                tc_fence_after();
                const uint32_t a_base = smem_u32(smem + static_cast<size_t>(st) * g.stage_bytes);
                const uint32_t b_base = a_base + g.a_block_bytes;
                const bool last = (c == g.n_kc - 1);
                for (int t = 0; t < g.KBc; ++t) {
                    const int grp = (c + 1 + t) % g.KBc;
                    if (grp >= g.G) continue;
                    if (c >= 1 && grp == c % g.KBc) {
                        if (!mbar_wait(&gempty[grp], static_cast<uint32_t>((ephase >> grp) & 1ull), vabort, TO)) {
                            ok = false;
                            break;
                        }
                        ephase ^= (1ull << grp);
                        tc_fence_after();
                    }
                    const int glo = max(g.grp_lo[grp], g.bin_lo), ghi = min(g.grp_hi[grp], g.bin_hi);
                    for (int kk = 0; kk < (g.KC >> 4); ++kk) {
                        for (int p = 0; p < g.s; ++p) {
                            const int jlo = max(glo, p), jhi = min(ghi, p + g.s - 1);
                            for (int j0 = jlo; j0 <= jhi; j0 += MAXB) {
                                const int j1 = min(jhi, j0 + MAXB - 1);
                                const int n = (j1 - j0 + 1) * BN;
                                const uint64_t ad = smem_desc(a_base + p * a_slice_bytes + kk * 256, 128, sbo);
                                const uint64_t bd =
                                    smem_desc(b_base + (j0 - p) * b_slice_bytes + kk * 256, 128, sbo);
                                umma_bf16(tmem + static_cast<uint32_t>(j0 * BN), ad, bd,
                                          idesc_base | (static_cast<uint32_t>(n >> 3) << 17), 1u);
                            }
                        }
                    }
                    if (((c + 1) % g.KBc) == grp || last) umma_commit(&gfull[grp]);
                }
                if (!ok) break;
                umma_commit(&empty[st]);
            }
            if (!ok && !*vabort) {
                atomicCAS(g.err, 0, DEVERR_TIMEOUT_MMA);
                *vabort = 1;
            }
            // all MMAs issued by this thread complete before TMEM is released
            umma_commit(mma_done);
            const int zero = 0;
            mbar_wait(mma_done, 0, &zero, TO);
        }
        __syncwarp();
    } else {
        // ------------------------------------------ drain + epilogue warps
        const int ew = warp - 2;
        const int qd = warp & 3;  // TMEM lane quadrant accessible to this warp
        const int half = ew >> 2;
        const uint32_t trow = tmem + (static_cast<uint32_t>(32 * qd) << 16) + static_cast<uint32_t>(half * HALF);

        for (int j = 0; j < g.J; ++j)
#pragma unroll
            for (int l = 0; l < NLD; ++l) tmem_st8_zero(trow + j * BN + l * 8);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tmem_ready);

        uint32_t q[HALF][W];
#pragma unroll
        for (int i = 0; i < HALF; ++i)
#pragma unroll
            for (int w = 0; w < W; ++w) q[i][w] = 0;

        uint64_t fphase = 0;
        bool ok = true;
        for (int c = 0; ok && c < g.n_kc; ++c) {
            const bool last = (c == g.n_kc - 1);
            const int ngr = last ? g.KBc : 1;
            for (int t = 0; t < ngr; ++t) {
                const int grp = (c + 1 + t) % g.KBc;
                if (grp >= g.G) continue;
                if (!mbar_wait(&gfull[grp], static_cast<uint32_t>((fphase >> grp) & 1ull), vabort, TO)) {
                    ok = false;
                    break;
                }
                fphase ^= (1ull << grp);
                tc_fence_after();
                const int glo = max(g.grp_lo[grp], g.bin_lo), ghi = min(g.grp_hi[grp], g.bin_hi);
                for (int j = glo; j <= ghi; ++j) {
                    const int sh = g.b * (g.J - 1 - j);
#pragma unroll
                    for (int cb = 0; cb < HALF / DB; ++cb) {
                        uint32_t v[DB];
#pragma unroll
                        for (int l = 0; l < DB / 8; ++l) tmem_ld8(trow + j * BN + cb * DB + l * 8, v + l * 8);
                        tmem_ld_wait();
#pragma unroll
                        for (int i = 0; i < DB; ++i) reg_fence(v[i]);
                        if (!last) {
#pragma unroll
                            for (int l = 0; l < DB / 8; ++l) tmem_st8_zero(trow + j * BN + cb * DB + l * 8);
                        }
                        q_add_shifted<W, DB>(q + cb * DB, v, sh);
                    }
                }
                if (!last) {
                    tmem_st_wait();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&gempty[grp]);
                }
            }
        }
        if (!ok && !*vabort) {
            atomicCAS(g.err, 0, DEVERR_TIMEOUT_EPI);
            *vabort = 1;
        }

        // ------------------------------------------------------- epilogue
        if (ok) {
            const int row = mt * BM + 32 * qd + lane;
            const int col0 = nt * BN + half * HALF;
            if (row < g.M) {
                const int er = g.er[row];
                const int bJ1 = g.b * (g.J + 1);
                if (g.out_mode == OUT_RAW) {
#pragma unroll
                    for (int i = 0; i < HALF; ++i) {
                        const int col = col0 + i;
                        if (col < g.N) {
                            int32_t *dst = g.raw + (static_cast<size_t>(row) * g.N + col) * 4;
                            const uint32_t ext = static_cast<uint32_t>(static_cast<int32_t>(q[i][W - 1]) >> 31);
#pragma unroll
                            for (int w = 0; w < 4; ++w) dst[w] = static_cast<int32_t>(w < W ? q[i][w] : ext);
                        }
                    }
                } else {
                    double *crow = g.c + static_cast<size_t>(row) * g.ldc;
#pragma unroll
                    for (int i = 0; i < HALF; ++i) {
                        const int col = col0 + i;
                        if (col < g.N) crow[col] = q_to_double<W>(q[i], er + g.ec[col], bJ1, g.out_mode);
                    }
                }
            }
        }
    }

    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, g.tmem_cols);
    }
}

template <int BN, int W>
void launch_gemm_variant(const GemmArgs &args, int grid, size_t smem, void *stream) {
    auto kern = oz_gemm_kernel<BN, W>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    kern<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(args);
}

}  // namespace ozgb
