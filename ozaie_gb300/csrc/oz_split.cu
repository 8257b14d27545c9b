// oz_split.cu -- stages (a) and (b): per-row / per-column maximum exponent and the
// error-free split of FP64 values into signed b-bit slices.
//
// Reference semantics (atlarge-research/ozAIE, src/aie_kernels/generic/ozaki_base.cc):
//   (a) ozaki_get_max_exponent_inner_tiled_wise_half_half  :342-440  (max of bits 52..62, start 0)
//   (b) extract_splits_acc64_half_half                     :449-639  (see split_value below)
// All work on the FP64 bit patterns is integer; FP64 arithmetic appears only in
// the optional sum of squares that the precision knob reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "oz_internal.h"
#include "oz_plan.h"
#include "oz_ptx.cuh"

namespace ozgb {

__device__ __forceinline__ int exp_field(double x) {
    return static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(x)) >> 52) & 0x7FF);
}

// ------------------------------------------------------------- stage (a)
// One warp per row of A: max exponent field (and sum of squares when ss != null).
__device__ __forceinline__ void rowmax_body(const double *__restrict__ A, long lda, int M, int K, int32_t *__restrict__ er,
                         double *__restrict__ ss, int bx, int by) {
    const int warp = (bx * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= M) return;
    const double *row = A + static_cast<size_t>(warp) * lda;
    int e = 0;
    double s2 = 0.0;
    for (int k = lane; k < K; k += 32) {
        const double x = __ldg(row + k);
        e = max(e, exp_field(x));
        if (ss) s2 = fma(x, x, s2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
        if (ss) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
        if (er) er[warp] = e;
        if (ss) ss[warp] = s2;
    }
}
__global__ void k_rowmax(const double *__restrict__ A, long lda, int M, int K, int32_t *__restrict__ er,
                         double *__restrict__ ss) {
    rowmax_body(A, lda, M, K, er, ss, blockIdx.x, blockIdx.y);
}

// One thread per column of B over a slab of rows; combined with atomicMax
// (ec must be zeroed first) and, when ss != null, atomicAdd of squares.
__device__ __forceinline__ void colmax_body(const double *__restrict__ B, long ldb, int K, int N, int rows_per_slab,
                         int32_t *__restrict__ ec, double *__restrict__ ss, int bx, int by) {
    const int n = bx * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int k0 = by * rows_per_slab;
    const int k1 = min(K, k0 + rows_per_slab);
    int e = 0;
    double s2 = 0.0;
    for (int k = k0; k < k1; ++k) {
        const double x = __ldg(B + static_cast<size_t>(k) * ldb + n);
        e = max(e, exp_field(x));
        if (ss) s2 = fma(x, x, s2);
    }
    if (ec) atomicMax(ec + n, e);
    if (ss) atomicAdd(ss + n, s2);
}
__global__ void k_colmax(const double *__restrict__ B, long ldb, int K, int N, int rows_per_slab,
                         int32_t *__restrict__ ec, double *__restrict__ ss) {
    colmax_body(B, ldb, K, N, rows_per_slab, ec, ss, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------- stage (b)
// The reference's split of one double (ozaki_base.cc:497-628), restated:
//   bias = E - e (uint32), mantissa with implicit one for normal numbers only,
//   m64 = mant << 11 (MSB at bit 63), words w0..w3 selected by bias >= 32/64/96
//   (w3 not cleared for bias >= 128 when two 64-bit windows are used),
//   X = (w0:w1:w2:w3) >> (bias mod 32),
//   slice_i = sign * ((X >> (128 - b(i+1))) & (2^b - 1)).
struct SplitState {
    unsigned __int128 X;
    bool neg;
};

__device__ __forceinline__ SplitState split_value(double x, int E, bool two_windows) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t e = static_cast<uint32_t>((u >> 52) & 0x7FF);
    const unsigned long long mant = (u & ((1ull << 52) - 1)) | (e ? (1ull << 52) : 0ull);
    const uint32_t bias = static_cast<uint32_t>(E) - e;
    const unsigned long long m64 = mant << 11;
    const uint32_t vhi = static_cast<uint32_t>(m64 >> 32), vlo = static_cast<uint32_t>(m64);
    const uint32_t w0 = bias >= 32u ? 0u : vhi;
    const uint32_t w1 = bias >= 64u ? 0u : (bias >= 32u ? vhi : vlo);
    uint32_t w2 = 0, w3 = 0;
    if (two_windows) {
        w2 = bias >= 96u ? 0u : (bias >= 64u ? vhi : (bias >= 32u ? vlo : 0u));
        w3 = bias >= 96u ? vhi : (bias >= 64u ? vlo : 0u);
    }
    const unsigned __int128 W = (static_cast<unsigned __int128>((static_cast<unsigned long long>(w0) << 32) | w1)
                                 << 64) |
                                static_cast<unsigned __int128>((static_cast<unsigned long long>(w2) << 32) | w3);
    SplitState st;
    st.X = W >> (bias & 31u);
    st.neg = (u >> 63) != 0;
    return st;
}

// The split window as four 32-bit words, most significant first (w[4] = 0 so that
// a slice straddling two words is one funnel shift), and the bf16 sign bit.
__device__ __forceinline__ void split_words(const SplitState &st, uint32_t (&w)[5], uint32_t &sign) {
    w[0] = static_cast<uint32_t>(st.X >> 96);
    w[1] = static_cast<uint32_t>(st.X >> 64);
    w[2] = static_cast<uint32_t>(st.X >> 32);
    w[3] = static_cast<uint32_t>(st.X);
    w[4] = 0u;
    sign = st.neg ? 0x8000u : 0u;
}

// bf16 bits of slice p (b = B bits at bit position B*p from the top), signed:
// the magnitude v < 2^8 becomes a float through the FP32 adder (2^23 + v - 2^23,
// exact) rather than the slower integer conversion; +0 for zero slices.
template <int B>
__device__ __forceinline__ uint32_t slice_bits(const uint32_t (&w)[5], uint32_t sign, int p) {
    const int pos = B * p;
    const int idx = pos >> 5, off = pos & 31;
    const uint32_t v = __funnelshift_l(w[idx + 1], w[idx], off) >> (32 - B);
    const uint32_t mag = __float_as_uint(__uint_as_float(0x4B000000u | v) - 8388608.0f) >> 16;
    return mag | (v ? sign : 0u);
}

// Four slices p of four elements as e4m3 bytes (element 0 in the lowest byte):
// every magnitude is < 16, so the conversion is exact.
template <int B>
__device__ __forceinline__ float slice_float(const uint32_t (&w)[5], uint32_t sign, int p) {
    const int pos = B * p;
    const int idx = pos >> 5, off = pos & 31;
    const uint32_t v = __funnelshift_l(w[idx + 1], w[idx], off) >> (32 - B);
    const float f = __uint_as_float(0x4B000000u | v) - 8388608.0f;
    return sign ? -f : f;
}
template <int B>
__device__ __forceinline__ uint32_t slices_e4m3x4(const uint32_t (*w)[5], const uint32_t *sg, int p) {
    uint16_t lo, hi;
    asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;"
        : "=h"(lo)
        : "f"(slice_float<B>(w[1], sg[1], p)), "f"(slice_float<B>(w[0], sg[0], p)));
    asm("cvt.rn.satfinite.e4m3x2.f32 %0, %1, %2;"
        : "=h"(hi)
        : "f"(slice_float<B>(w[3], sg[3], p)), "f"(slice_float<B>(w[2], sg[2], p)));
    return static_cast<uint32_t>(lo) | (static_cast<uint32_t>(hi) << 16);
}

// One-window split (s b within the first window, see split_two_windows): the
// slices are then the top s b bits of V = (mantissa << 11) >> bias (0 for
// bias >= 64), the same bits as split_value's 128-bit window, whose low 64 bits
// hold no slice.  V is kept as two words plus the element's sign in the two
// forms the bf16 conversion below uses.
struct FastElem {
    uint32_t hi, lo;  // V
    uint32_t sgnc;    // 0x4B000000 with the sign bit of x
    float cadd;       // -2^23 for x >= 0, +2^23 for x < 0
};
__device__ __forceinline__ FastElem fast_elem(double x, int E) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const uint32_t e = static_cast<uint32_t>((u >> 52) & 0x7FF);
    const unsigned long long mant = (u & ((1ull << 52) - 1)) | (e ? (1ull << 52) : 0ull);
    const uint32_t bias = static_cast<uint32_t>(E) - e;
    const unsigned long long v = bias < 64u ? (mant << 11) >> bias : 0ull;
    const uint32_t neg = static_cast<uint32_t>(u >> 63);
    FastElem r;
    r.hi = static_cast<uint32_t>(v >> 32);
    r.lo = static_cast<uint32_t>(v);
    r.sgnc = 0x4B000000u | (neg << 31);
    r.cadd = neg ? 8388608.0f : -8388608.0f;
    return r;
}
// Slice p (B bits at bit B*p from the top of V) as a signed float: the FP32
// bits of +-(2^23 + v) plus -+2^23 give +-v exactly (and +0 for v = 0): one
// shift, one three-input logic operation and one add.
template <int B>
__device__ __forceinline__ float fast_slice(const FastElem &x, int p) {
    const int sh = 64 - B * (p + 1);  // V >> sh puts the slice in the low bits
    const uint32_t f = sh >= 32 ? (x.hi >> (sh - 32)) : __funnelshift_r(x.lo, x.hi, sh);
    return __uint_as_float((f & ((1u << B) - 1u)) | x.sgnc) + x.cadd;
}
// Two floats holding integers of magnitude < 256 as bf16 (exact): lo in bits 0..15.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
// 16 bytes of slice p: 8 consecutive K values of one row, as bf16.
template <int B>
__device__ __forceinline__ uint4 fast_slice8(const FastElem (&x)[8], int p) {
    uint4 v;
    v.x = pack_bf16x2(fast_slice<B>(x[0], p), fast_slice<B>(x[1], p));
    v.y = pack_bf16x2(fast_slice<B>(x[2], p), fast_slice<B>(x[3], p));
    v.z = pack_bf16x2(fast_slice<B>(x[4], p), fast_slice<B>(x[5], p));
    v.w = pack_bf16x2(fast_slice<B>(x[6], p), fast_slice<B>(x[7], p));
    return v;
}

__host__ __device__ inline bool split_two_windows(int b, int s) {
    const int avoid = 1 + (b == 3 ? 3 : 0);
    const int nv0 = 64 - avoid - ((64 - avoid) % b);
    return s * b > nv0;
}

// A [M][K] row-major -> A slice blocks [mt][c][p][128 x KC].  One thread takes 8
// consecutive K values of one row and writes one 16-byte piece per slice; a warp
// covers 8 rows x 32 K (4 core matrices of each slice, 512 contiguous bytes).
template <int B, bool F8 = false>
__device__ __forceinline__ void split_a_body(const double *__restrict__ A, long lda, int M, int K,
                                             const int32_t *__restrict__ er, int s, int KC, int n_kc, int Mp,
                                             uint16_t *__restrict__ tiles, int bx, int by, bool trans) {
    const int r8 = threadIdx.x & 7;
    const int kgl = threadIdx.x >> 3;  // 0..31
    const int m = by * 8 + r8;
    const int k0 = (bx * 32 + kgl) * 8;
    const int Kp = n_kc * KC;
    if (m >= Mp || k0 >= Kp) return;
    const bool two = split_two_windows(B, s);
    const int E = m < M ? er[m] : 0;
    const double *row = A + static_cast<size_t>(m) * lda;
    if (!F8 && !two) {
        // one window: 128-bit loads where the row's 8 values are in range and
        // aligned, the shift-and-add slice conversion
        double xv[8];
        const double *src = row + k0;
        if (!trans && m < M && k0 + 8 <= K && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const double2 d = __ldg(reinterpret_cast<const double2 *>(src) + i);
                xv[2 * i] = d.x;
                xv[2 * i + 1] = d.y;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int k = k0 + i;
                xv[i] = (m < M && k < K) ? __ldg(trans ? A + static_cast<size_t>(k) * lda + m : row + k) : 0.0;
            }
        }
        FastElem fe[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) fe[i] = fast_elem(xv[i], E);
        const int mt = m >> 7, r = m & 127, c = k0 / KC, kk = k0 % KC;
        const size_t slice_elems = static_cast<size_t>(BM) * KC;
        uint16_t *dst = tiles + (static_cast<size_t>(mt) * n_kc + c) * s * slice_elems + canon_offset(r, kk, KC);
#pragma unroll
        for (int p = 0; p < 64 / B; ++p)
            if (p < s) *reinterpret_cast<uint4 *>(dst + p * slice_elems) = fast_slice8<B>(fe, p);
        return;
    }
    uint32_t w[8][5], sg[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int k = k0 + i;
        const double x = (m < M && k < K) ? __ldg(trans ? A + static_cast<size_t>(k) * lda + m : row + k) : 0.0;
        split_words(split_value(x, E, two), w[i], sg[i]);
    }
    const int mt = m >> 7, r = m & 127, c = k0 / KC, kk = k0 % KC;
    const size_t slice_elems = static_cast<size_t>(BM) * KC;
    if constexpr (F8) {
        // one-byte slices: 8 bytes per thread and slice
        uint8_t *dst8 = reinterpret_cast<uint8_t *>(tiles) + (static_cast<size_t>(mt) * n_kc + c) * s * slice_elems +
                        canon_offset8(r, kk, KC);
#pragma unroll
        for (int p = 0; p < 128 / B; ++p) {
            if (p < s) {
                uint2 v;
                v.x = slices_e4m3x4<B>(w, sg, p);
                v.y = slices_e4m3x4<B>(w + 4, sg + 4, p);
                *reinterpret_cast<uint2 *>(dst8 + p * slice_elems) = v;
            }
        }
        return;
    }
    uint16_t *dst = tiles + (static_cast<size_t>(mt) * n_kc + c) * s * slice_elems + canon_offset(r, kk, KC);
#pragma unroll
    for (int p = 0; p < 128 / B; ++p) {
        if (p < s) {
            uint4 v;
            v.x = slice_bits<B>(w[0], sg[0], p) | (slice_bits<B>(w[1], sg[1], p) << 16);
            v.y = slice_bits<B>(w[2], sg[2], p) | (slice_bits<B>(w[3], sg[3], p) << 16);
            v.z = slice_bits<B>(w[4], sg[4], p) | (slice_bits<B>(w[5], sg[5], p) << 16);
            v.w = slice_bits<B>(w[6], sg[6], p) | (slice_bits<B>(w[7], sg[7], p) << 16);
            *reinterpret_cast<uint4 *>(dst + p * slice_elems) = v;
        }
    }
}
template <int B, bool F8>
__global__ void k_split_a(const double *__restrict__ A, long lda, int M, int K, const int32_t *__restrict__ er,
                          int s, int KC, int n_kc, int Mp, uint16_t *__restrict__ tiles, int trans) {
    split_a_body<B, F8>(A, lda, M, K, er, s, KC, n_kc, Mp, tiles, blockIdx.x, blockIdx.y, trans != 0);
}

// B [K][N] row-major -> slice blocks of B^T [nt][c][q][BN x KC].  One thread
// takes one column n and 8 consecutive K; a warp reads 32 consecutive columns
// per row (coalesced) and writes four 128-byte core matrices per slice.
template <int B, bool F8 = false>
__device__ __forceinline__ void split_b_body(const double *__restrict__ Bm, long ldb, int K, int N,
                                             const int32_t *__restrict__ ec, int s, int KC, int n_kc, int BN, int Np,
                                             uint16_t *__restrict__ tiles, int bx, int by, bool trans) {
    const int n = bx * 32 + (threadIdx.x & 31);
    const int k0 = (by * 8 + (threadIdx.x >> 5)) * 8;
    const int Kp = n_kc * KC;
    if (n >= Np || k0 >= Kp) return;
    const bool two = split_two_windows(B, s);
    const int E = n < N ? ec[n] : 0;
    if (!F8 && !two) {
        // one window: the shift-and-add slice conversion
        FastElem fe[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int k = k0 + i;
            const double x = (n < N && k < K) ? __ldg(trans ? Bm + static_cast<size_t>(n) * ldb + k
                                                            : Bm + static_cast<size_t>(k) * ldb + n)
                                              : 0.0;
            fe[i] = fast_elem(x, E);
        }
        const int nt = n / BN, r = n % BN, c = k0 / KC, kk = k0 % KC;
        const size_t slice_elems = static_cast<size_t>(BN) * KC;
        uint16_t *dst = tiles + (static_cast<size_t>(nt) * n_kc + c) * s * slice_elems + canon_offset(r, kk, KC);
#pragma unroll
        for (int q = 0; q < 64 / B; ++q)
            if (q < s) *reinterpret_cast<uint4 *>(dst + q * slice_elems) = fast_slice8<B>(fe, q);
        return;
    }
    uint32_t w[8][5], sg[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int k = k0 + i;
        const double x =
            (n < N && k < K) ? __ldg(trans ? Bm + static_cast<size_t>(n) * ldb + k : Bm + static_cast<size_t>(k) * ldb + n)
                             : 0.0;
        split_words(split_value(x, E, two), w[i], sg[i]);
    }
    const int nt = n / BN, r = n % BN, c = k0 / KC, kk = k0 % KC;
    const size_t slice_elems = static_cast<size_t>(BN) * KC;
    if constexpr (F8) {
        uint8_t *dst8 = reinterpret_cast<uint8_t *>(tiles) + (static_cast<size_t>(nt) * n_kc + c) * s * slice_elems +
                        canon_offset8(r, kk, KC);
#pragma unroll
        for (int q = 0; q < 128 / B; ++q) {
            if (q < s) {
                uint2 v;
                v.x = slices_e4m3x4<B>(w, sg, q);
                v.y = slices_e4m3x4<B>(w + 4, sg + 4, q);
                *reinterpret_cast<uint2 *>(dst8 + q * slice_elems) = v;
            }
        }
        return;
    }
    uint16_t *dst = tiles + (static_cast<size_t>(nt) * n_kc + c) * s * slice_elems + canon_offset(r, kk, KC);
#pragma unroll
    for (int q = 0; q < 128 / B; ++q) {
        if (q < s) {
            uint4 v;
            v.x = slice_bits<B>(w[0], sg[0], q) | (slice_bits<B>(w[1], sg[1], q) << 16);
            v.y = slice_bits<B>(w[2], sg[2], q) | (slice_bits<B>(w[3], sg[3], q) << 16);
            v.z = slice_bits<B>(w[4], sg[4], q) | (slice_bits<B>(w[5], sg[5], q) << 16);
            v.w = slice_bits<B>(w[6], sg[6], q) | (slice_bits<B>(w[7], sg[7], q) << 16);
            *reinterpret_cast<uint4 *>(dst + q * slice_elems) = v;
        }
    }
}
template <int B, bool F8>
__global__ void k_split_b(const double *__restrict__ Bm, long ldb, int K, int N, const int32_t *__restrict__ ec,
                          int s, int KC, int n_kc, int BN, int Np, uint16_t *__restrict__ tiles, int trans) {
    split_b_body<B, F8>(Bm, ldb, K, N, ec, s, KC, n_kc, BN, Np, tiles, blockIdx.x, blockIdx.y, trans != 0);
}

// b (1..7) as a template argument: the slice positions become constants.
#define OZ_SPLIT_DISPATCH(b, CALL) \
    switch (b) {                   \
        case 1: CALL(1); break;    \
        case 2: CALL(2); break;    \
        case 3: CALL(3); break;    \
        case 4: CALL(4); break;    \
        case 5: CALL(5); break;    \
        case 6: CALL(6); break;    \
        default: CALL(7); break;   \
    }
// b <= 4 (the e4m3 carrier holds |v| <= 15 exactly)
#define OZ_SPLIT_DISPATCH_F8(b, CALL) \
    switch (b) {                      \
        case 1: CALL(1); break;       \
        case 2: CALL(2); break;       \
        case 3: CALL(3); break;       \
        default: CALL(4); break;      \
    }

// A kernel whose only wait is on an mbarrier that nothing arrives on: exercises
// the bounded-wait path (records DEVERR_TIMEOUT_SELFTEST and returns).
__global__ void k_selftest_timeout(int *err, unsigned long long timeout_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int zero = 0;
        if (!mbar_wait(&bar, 0, &zero, timeout_ns)) atomicCAS(err, 0, DEVERR_TIMEOUT_SELFTEST);
    }
}

// Block-wide reductions over blockDim.x threads (a multiple of 32, at most 1024).
__device__ int block_max_int(int v, int *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int m = sh[0];
    for (int w = 1; w < nw; ++w) m = max(m, sh[w]);
    return m;
}

__device__ double block_max_nonneg(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double m = sh[0];
    for (int w = 1; w < nw; ++w) m = fmax(m, sh[w]);
    return m;
}

__device__ double block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += sh[w];
    return s;
}

// Precision-knob statistics, all scaled by the largest row exponent ea of A and
// the largest column exponent eb of B so that they stay in range:
//   out[0] = sum_i 4^{Er_i-ea}           out[1] = sum_i |a_i|^2 4^{1022-ea}
//   out[2] = sum_j 4^{Ec_j-eb}           out[3] = sum_j |b_j|^2 4^{1022-eb}
//   out[4] = sum_k |A(:,k)|^2 |B(k,:)|^2 4^{2044-ea-eb}
// Block 0 makes the A terms, block 1 the B terms, block 2 the K-direction term.
// 2^e as an exact double for e in [-1022, 1023] (0 below: those terms are
// negligible in the knob's sums).
__device__ __forceinline__ double pow2i(int e) {
    if (e < -1022) return 0.0;
    return __longlong_as_double(static_cast<long long>(min(e, 1023) + 1023) << 52);
}
// x * 2^e for e in [-2046, 2046], as two exact power-of-two products.
__device__ __forceinline__ double scale2(double x, int e) {
    const int h = e / 2;
    return x * pow2i(h) * pow2i(e - h);
}

// ------------------------------------------------ FP32 scaled sums of squares
// 4^d as a float for d <= 0 (0 below the normal range).
__device__ __forceinline__ float pow4f(int d) { return d < -63 ? 0.0f : __int_as_float((127 + 2 * d) << 23); }

// (E, s) += the square of x: s is in units of 4^(E-1023), E the largest exponent
// field seen; x's own mantissa m in [1, 2) squared is added at 4^(e-E).
__device__ __forceinline__ void sq_add(int &E, float &s, double x) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const int e = static_cast<int>((u >> 52) & 0x7FF);
    if (e == 0 || e == 0x7FF) return;  // zeros and subnormals (negligible); no infinities
    const float m = __uint_as_float(0x3F800000u | static_cast<uint32_t>((u >> 29) & 0x7FFFFF));
    if (e > E) {
        s *= pow4f(E - e);
        E = e;
    }
    s = fmaf(m * m, pow4f(e - E), s);
}
__device__ __forceinline__ void sq_merge(int &E, float &s, int E2, float s2) {
    const int Em = max(E, E2);
    s = s * pow4f(E - Em) + s2 * pow4f(E2 - Em);
    E = Em;
}
__device__ __forceinline__ unsigned long long sq_pack(int E, float s) {
    return (static_cast<unsigned long long>(static_cast<uint32_t>(E)) << 32) | __float_as_uint(s);
}

// (E, s) += m2 * 4^(e - 1023) for an element with exponent field e and squared
// mantissa m2 (0 for zeros, subnormals and non-finite values).
__device__ __forceinline__ void sq_add_em(int &E, float &s, int e, float m2) {
    if (e > E) {
        s *= pow4f(E - e);
        E = e;
    }
    s = fmaf(m2, pow4f(e - E), s);
}

// One 64-row x 256-column tile.  Lane l of each warp owns the 8 columns
// bx*256 + l + 32k (each load instruction of a warp reads 256 contiguous bytes)
// and warp w the rows w, w+8, ..., so a row is reduced by the
// warp's shuffles alone (no block barrier in the row loop); the 8 warps' column
// partials are merged once through shared memory at the end.
__device__ __forceinline__ void stats2d_body(const double *__restrict__ X, long ld, int rows, int cols,
                                             int32_t *__restrict__ row_e, int32_t *__restrict__ col_e,
                                             unsigned long long *__restrict__ row_part,
                                             unsigned long long *__restrict__ col_part, int bx, int by) {
    constexpr int NW = kStageThreads / 32;           // warps per block
    constexpr int CPL = kStatsCols / 32;             // columns per lane (8)
    static_assert(CPL == 8 && kStatsRows % NW == 0, "stats tile");
    __shared__ int shE[NW][kStatsCols];
    __shared__ float shS[NW][kStatsCols];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int c0 = bx * kStatsCols + lane;            // this lane's first column; then every 32nd
    const int r0 = by * kStatsRows;
    const bool rows_wanted = row_e || row_part;
    const int nbx = (cols + kStatsCols - 1) / kStatsCols;
    int Ec[CPL];
    float sc[CPL];
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
        Ec[k] = 0;
        sc[k] = 0.0f;
    }
    auto load_row = [&](int r, double (&x)[CPL]) {
#pragma unroll
        for (int k = 0; k < CPL; ++k)
            x[k] = (r < rows && c0 + 32 * k < cols) ? __ldg(X + static_cast<size_t>(r) * ld + c0 + 32 * k) : 0.0;
    };
    // the next row's loads are issued before this row is reduced
    double x[CPL], xn[CPL];
    if (wid < kStatsRows) load_row(r0 + wid, xn);
    for (int i = wid; i < kStatsRows; i += NW) {
        const int r = r0 + i;
#pragma unroll
        for (int k = 0; k < CPL; ++k) x[k] = xn[k];
        if (i + NW < kStatsRows) load_row(r + NW, xn);
        int ex[CPL];
        uint32_t mb[CPL];  // FP32 mantissa bits of each element; 0 for zeros, subnormals, non-finite
        int Er = 0;
#pragma unroll
        for (int k = 0; k < CPL; ++k) {
            const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x[k]));
            ex[k] = static_cast<int>((bits >> 52) & 0x7FF);
            mb[k] = (ex[k] != 0 && ex[k] != 0x7FF) ? (0x800000u | static_cast<uint32_t>((bits >> 29) & 0x7FFFFF)) : 0u;
            Er = max(Er, ex[k]);
        }
        // columns: running exponent per column, rescaled only when a larger one
        // appears (rare after the first rows); x scaled by 2^(-Ec) squared by one FMA
#pragma unroll
        for (int k = 0; k < CPL; ++k) {
            if (ex[k] > Ec[k]) {
                sc[k] *= pow4f(Ec[k] - ex[k]);
                Ec[k] = ex[k];
            }
            const int d = ex[k] - Ec[k];
            const float xs = (mb[k] && d >= -63) ? __uint_as_float((static_cast<uint32_t>(d + 127) << 23) |
                                                                   (mb[k] & 0x7FFFFFu))
                                                 : 0.0f;
            sc[k] = fmaf(xs, xs, sc[k]);
        }
        if (rows_wanted) {
            // rows: one exponent for the whole row (the warp's maximum), then plain sums
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) Er = max(Er, __shfl_xor_sync(0xffffffffu, Er, o));
            float sr = 0.0f;
#pragma unroll
            for (int k = 0; k < CPL; ++k) {
                const int d = ex[k] - Er;
                const float xs = (mb[k] && d >= -63) ? __uint_as_float((static_cast<uint32_t>(d + 127) << 23) |
                                                                       (mb[k] & 0x7FFFFFu))
                                                     : 0.0f;
                sr = fmaf(xs, xs, sr);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sr += __shfl_xor_sync(0xffffffffu, sr, o);
            if (lane == 0 && r < rows) {
                if (row_part) row_part[static_cast<size_t>(r) * nbx + bx] = sq_pack(Er, sr);
                if (row_e) atomicMax(row_e + r, Er);
            }
        }
    }
    // columns: merge the warps' partials
#pragma unroll
    for (int k = 0; k < CPL; ++k) {
        shE[wid][lane + 32 * k] = Ec[k];
        shS[wid][lane + 32 * k] = sc[k];
    }
    __syncthreads();
    const int c = bx * kStatsCols + static_cast<int>(threadIdx.x);
    if (c < cols) {
        int E = 0;
        float sv = 0.0f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sq_merge(E, sv, shE[w][threadIdx.x], shS[w][threadIdx.x]);
        if (col_part) col_part[static_cast<size_t>(by) * cols + c] = sq_pack(E, sv);
        if (col_e) atomicMax(col_e + c, E);
    }
}


// Combined (E, s) of unit u, by one warp: lanes load the unit's partials in
// parallel and merge them; every lane returns the result.
__device__ __forceinline__ void unit_sq_warp(const StatParts &sp, int u, int lane, int *E, float *s) {
    int e = 0;
    float v = 0.0f;
    const unsigned long long *p = sp.p + u * sp.unit_stride;
    for (int i = lane; i < sp.nparts; i += 32) {
        const unsigned long long w = __ldg(p + i * sp.part_stride);
        sq_merge(e, v, static_cast<int>(w >> 32), __uint_as_float(static_cast<uint32_t>(w)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int e2 = __shfl_xor_sync(0xffffffffu, e, o);
        const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        sq_merge(e, v, e2, v2);
    }
    *E = e;
    *s = v;
}

// Combined (E, s) of unit u by one thread, for units with few partials: the
// loads of many units are in flight at once instead of one unit per warp.
__device__ __forceinline__ void unit_sq_thread(const StatParts &sp, int u, int *E, float *s) {
    int e = 0;
    float v = 0.0f;
    const unsigned long long *p = sp.p + u * sp.unit_stride;
#pragma unroll 4
    for (int i = 0; i < sp.nparts; ++i) {
        const unsigned long long w = __ldg(p + i * sp.part_stride);
        sq_merge(e, v, static_cast<int>(w >> 32), __uint_as_float(static_cast<uint32_t>(w)));
    }
    *E = e;
    *s = v;
}

// Part `chunk` of `chunks` of one of the three knob sums (role 0: A terms, 1: B
// terms, 2: the k-direction term), added atomically into j.out (zeroed before);
// one warp per unit.  With ea, eb the largest row / column exponents of op(A) /
// op(B):
//   sa = sum_r 4^(Er - ea), na = sum_r |a_r|^2 4^(1022 - ea), likewise for B,
//   t  = sum_k |op(A)(:,k)|^2 |op(B)(k,:)|^2 4^(2044 - ea - eb),
// and for the elementwise criterion ia = max_r 1 / (|a_r|^2 4^(1022 - Er)) over
// the non-zero rows (ib likewise over the columns of op(B)), combined by an
// integer max of the bit patterns (order-preserving for non-negative doubles).
__device__ __forceinline__ void knob_stats_body(const KnobJob &j, const int role, const int chunk, const int chunks) {
    __shared__ int sh_i[32];
    __shared__ double sh_d[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int ea = 0, eb = 0;
    if (role != 1) {
        for (int i = threadIdx.x; i < j.M; i += blockDim.x) ea = max(ea, j.er[i]);
        ea = block_max_int(ea, sh_i);
    }
    if (role != 0) {
        for (int i = threadIdx.x; i < j.N; i += blockDim.x) eb = max(eb, j.ec[i]);
        eb = block_max_int(eb, sh_i);
    }
    const int n = role == 0 ? j.M : (role == 1 ? j.N : j.K);
    const int per = (n + chunks - 1) / chunks;
    const int i0 = chunk * per, i1 = min(n, i0 + per);
    double num = 0.0, den = 0.0, t = 0.0, inv = 0.0;
    // 1 / (|x_u|^2 4^(1022 - E_u)) of a unit whose squares sum to sq 4^(E - 1023)
    auto flat_inv = [](float sq, int E, int Eu) {
        return sq > 0.0f ? scale2(1.0 / static_cast<double>(sq), 2 * (Eu + 1 - E)) : 0.0;
    };
    const int nparts = role == 0 ? j.ra.nparts : (role == 1 ? j.cb.nparts : max(j.ka.nparts, j.kb.nparts));
    if (nparts <= 32) {
        // one thread per unit
        for (int u = i0 + static_cast<int>(threadIdx.x); u < i1; u += blockDim.x) {
            if (role < 2) {
                const StatParts &sp = role == 0 ? j.ra : j.cb;
                const int emax = role == 0 ? ea : eb;
                int E;
                float sq;
                unit_sq_thread(sp, u, &E, &sq);
                const int Eu = role == 0 ? j.er[u] : j.ec[u];
                num += pow2i(2 * (Eu - emax));
                den += scale2(static_cast<double>(sq), 2 * (E - emax) - 2);
                inv = fmax(inv, flat_inv(sq, E, Eu));
            } else {
                int E1, E2;
                float s1, s2;
                unit_sq_thread(j.ka, u, &E1, &s1);
                unit_sq_thread(j.kb, u, &E2, &s2);
                t += scale2(static_cast<double>(s1) * s2, 2 * (E1 + E2 - ea - eb - 2));
            }
        }
    } else {
        // one warp per unit
        for (int u = i0 + wid; u < i1; u += nw) {
            if (role < 2) {
                const StatParts &sp = role == 0 ? j.ra : j.cb;
                const int emax = role == 0 ? ea : eb;
                int E;
                float sq;
                unit_sq_warp(sp, u, lane, &E, &sq);
                if (lane == 0) {
                    const int Eu = role == 0 ? j.er[u] : j.ec[u];
                    num += pow2i(2 * (Eu - emax));
                    den += scale2(static_cast<double>(sq), 2 * (E - emax) - 2);
                    inv = fmax(inv, flat_inv(sq, E, Eu));
                }
            } else {
                int E1, E2;
                float s1, s2;
                unit_sq_warp(j.ka, u, lane, &E1, &s1);
                unit_sq_warp(j.kb, u, lane, &E2, &s2);
                if (lane == 0) t += scale2(static_cast<double>(s1) * s2, 2 * (E1 + E2 - ea - eb - 2));
            }
        }
    }
    if (role < 2) {
        num = block_sum(num, sh_d);
        den = block_sum(den, sh_d);
        inv = block_max_nonneg(inv, sh_d);
        if (threadIdx.x == 0) {
            atomicAdd(j.out + 2 * role, num);
            atomicAdd(j.out + 2 * role + 1, den);
            if (inv > 0.0)
                atomicMax(reinterpret_cast<unsigned long long *>(j.out + 5 + role),
                          static_cast<unsigned long long>(__double_as_longlong(inv)));
        }
    } else {
        t = block_sum(t, sh_d);
        if (threadIdx.x == 0) atomicAdd(j.out + 4, t);
    }
}

__global__ void k_knob_stats(const KnobJob j) { knob_stats_body(j, blockIdx.x % 3, blockIdx.x / 3, gridDim.x / 3); }

// Grouped knob reduction: blocks 3p, 3p+1, 3p+2 reduce problem p.
__global__ void k_knob_grouped(const KnobJob *__restrict__ jobs) {
    const KnobJob j = jobs[blockIdx.x / 3];
    knob_stats_body(j, blockIdx.x % 3, 0, 1);
}

// Grouped stage (a)/(b): block -> job by binary search over block0[], then the
// job's per-problem kernel body with its local block coordinates.
// One stage job on its local block index (the per-problem kernels' bodies).
// TRANS: the kernel also serves transposed splits (the grouped kernel does not,
// which keeps its register count down).
template <bool TRANS>
__device__ __forceinline__ void run_stage_job(const StageJob &j, int local) {
    const int bx = local % j.gx, by = local / j.gx;
    const bool tr = TRANS && j.trans != 0;
    switch (j.kind) {
        case JOB_ROWMAX: rowmax_body(j.X, j.ld, j.rows, j.cols, j.e_out, j.ss_out, bx, by); break;
        case JOB_COLMAX: colmax_body(j.X, j.ld, j.rows, j.cols, 64, j.e_out, j.ss_out, bx, by); break;
        case JOB_STATS: stats2d_body(j.X, j.ld, j.rows, j.cols, j.e_out, j.e_out2, j.prow, j.pcol, bx, by); break;
        // the transpose flag as a constant at each call site: a runtime flag would
        // compile both load paths into every split (measured 20 % slower)
        case JOB_SPLIT_A: {
#define OZ_JOB_A(BB, T) \
    split_a_body<BB>(j.X, j.ld, j.rows, j.cols, j.e_in, j.s, j.KC, j.n_kc, j.padded, j.tiles, bx, by, T)
#define OZ_JOB_A8(BB, T) \
    split_a_body<BB, true>(j.X, j.ld, j.rows, j.cols, j.e_in, j.s, j.KC, j.n_kc, j.padded, j.tiles, bx, by, T)
#define OZ_JOB_AN(BB) OZ_JOB_A(BB, false)
#define OZ_JOB_AT(BB) OZ_JOB_A(BB, true)
#define OZ_JOB_A8N(BB) OZ_JOB_A8(BB, false)
#define OZ_JOB_A8T(BB) OZ_JOB_A8(BB, true)
            if (j.f8) {
                if (tr) {
                    OZ_SPLIT_DISPATCH_F8(j.b, OZ_JOB_A8T)
                } else {
                    OZ_SPLIT_DISPATCH_F8(j.b, OZ_JOB_A8N)
                }
            } else {
                if (tr) {
                    OZ_SPLIT_DISPATCH(j.b, OZ_JOB_AT)
                } else {
                    OZ_SPLIT_DISPATCH(j.b, OZ_JOB_AN)
                }
            }
#undef OZ_JOB_A
#undef OZ_JOB_A8
#undef OZ_JOB_AN
#undef OZ_JOB_AT
#undef OZ_JOB_A8N
#undef OZ_JOB_A8T
            break;
        }
        default: {
#define OZ_JOB_B(BB, T) \
    split_b_body<BB>(j.X, j.ld, j.rows, j.cols, j.e_in, j.s, j.KC, j.n_kc, j.BN, j.padded, j.tiles, bx, by, T)
#define OZ_JOB_B8(BB, T) \
    split_b_body<BB, true>(j.X, j.ld, j.rows, j.cols, j.e_in, j.s, j.KC, j.n_kc, j.BN, j.padded, j.tiles, bx, by, T)
#define OZ_JOB_BN(BB) OZ_JOB_B(BB, false)
#define OZ_JOB_BT(BB) OZ_JOB_B(BB, true)
#define OZ_JOB_B8N(BB) OZ_JOB_B8(BB, false)
#define OZ_JOB_B8T(BB) OZ_JOB_B8(BB, true)
            if (j.f8) {
                if (tr) {
                    OZ_SPLIT_DISPATCH_F8(j.b, OZ_JOB_B8T)
                } else {
                    OZ_SPLIT_DISPATCH_F8(j.b, OZ_JOB_B8N)
                }
            } else {
                if (tr) {
                    OZ_SPLIT_DISPATCH(j.b, OZ_JOB_BT)
                } else {
                    OZ_SPLIT_DISPATCH(j.b, OZ_JOB_BN)
                }
            }
#undef OZ_JOB_B
#undef OZ_JOB_B8
#undef OZ_JOB_BN
#undef OZ_JOB_BT
#undef OZ_JOB_B8N
#undef OZ_JOB_B8T
            break;
        }
    }
}

// Persistent: block b runs work blocks b, b + gridDim.x, ... of the job list; the
// job of a work block is found by a forward scan from the previous one (work
// blocks only increase), so no block pays a search over all jobs, and a grouped
// call of many small problems does not launch one block per 2048 elements.
__global__ void __launch_bounds__(kStageThreads) k_stage_jobs(const StageJob *__restrict__ jobs,
                                                              const int *__restrict__ block0, int n_jobs) {
    const int total = __ldg(block0 + n_jobs);
    int j = 0;
    for (int bid = blockIdx.x; bid < total; bid += gridDim.x) {
        while (j + 1 < n_jobs && __ldg(block0 + j + 1) <= bid) ++j;
        run_stage_job<false>(jobs[j], bid - __ldg(block0 + j));
        // the statistics job's shared memory is written again by the next work block
        __syncthreads();
    }
}

// Two jobs of one problem (A and B) in one launch: blocks [0, n0) run j0.
__global__ void __launch_bounds__(kStageThreads) k_stage_pair(const __grid_constant__ StageJob j0,
                                                              const __grid_constant__ StageJob j1, int n0) {
    const int bid = blockIdx.x;
    if (bid < n0) run_stage_job<true>(j0, bid);
    else run_stage_job<true>(j1, bid - n0);
}

// Pseudo-random doubles in [-1, 1) (splitmix64 of the index): inputs for the
// autotuner's timing runs, whose speed does not depend on the values.
__global__ void k_fill_random(double *__restrict__ x, size_t n, unsigned long long seed) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        x[i] = static_cast<double>(z >> 11) * 0x1.0p-52 - 1.0;
    }
}

void launch_fill_random(double *x, size_t n, unsigned long long seed, void *stream) {
    if (n) k_fill_random<<<4 * 152, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, seed);
}

// C = beta * C over an M x N block with leading dimension ldc (beta == 0 writes
// zeros without reading C, as BLAS does).
__global__ void k_scale(double *__restrict__ C, long ldc, int M, int N, double beta) {
    const size_t total = static_cast<size_t>(M) * N;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        double *c = C + (i / N) * ldc + (i % N);
        *c = beta == 0.0 ? 0.0 : beta * *c;
    }
}

void launch_scale(double *C, long ldc, int M, int N, double beta, void *stream) {
    k_scale<<<4 * 152, 256, 0, static_cast<cudaStream_t>(stream)>>>(C, ldc, M, N, beta);
}

void stage_grid(const StageJob &j, int *gx, int *gy) {
    switch (j.kind) {
        case JOB_ROWMAX:
            *gx = (j.rows * 32 + kStageThreads - 1) / kStageThreads;
            *gy = 1;
            break;
        case JOB_COLMAX:
            *gx = (j.cols + kStageThreads - 1) / kStageThreads;
            *gy = (j.rows + 63) / 64;
            break;
        case JOB_STATS:
            *gx = (j.cols + kStatsCols - 1) / kStatsCols;
            *gy = (j.rows + kStatsRows - 1) / kStatsRows;
            break;
        case JOB_SPLIT_A:
            *gx = (j.n_kc * j.KC / 8 + 31) / 32;
            *gy = j.padded / 8;
            break;
        default:
            *gx = (j.padded + 31) / 32;
            *gy = (j.n_kc * j.KC / 8 + 7) / 8;
            break;
    }
}

void launch_stage_pair(StageJob j0, StageJob j1, void *stream) {
    stage_grid(j0, &j0.gx, &j0.gy);
    stage_grid(j1, &j1.gx, &j1.gy);
    const int n0 = j0.gx * j0.gy, n1 = j1.gx * j1.gy;
    if (n0 + n1 > 0)
        k_stage_pair<<<n0 + n1, kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(j0, j1, n0);
}

void launch_stage_jobs(const StageJob *jobs, const int *block0, int n_jobs, int total_blocks, void *stream) {
    if (total_blocks <= 0) return;
    // resident blocks of k_stage_jobs on the current device, found once per device
    static std::atomic<int> resident[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int grid = 0;
    if (dev >= 0 && dev < 64) grid = resident[dev].load(std::memory_order_relaxed);
    if (grid <= 0) {
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 148;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_jobs, kStageThreads, 0) != cudaSuccess ||
            per_sm <= 0)
            per_sm = 2;
        cudaGetLastError();
        grid = sms * per_sm;
        if (dev >= 0 && dev < 64) resident[dev].store(grid, std::memory_order_relaxed);
    }
    k_stage_jobs<<<std::min(grid, total_blocks), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(jobs, block0,
                                                                                                      n_jobs);
}

void launch_knob_grouped(const KnobJob *jobs, int n, void *stream) {
    if (n > 0) k_knob_grouped<<<3 * n, 256, 0, static_cast<cudaStream_t>(stream)>>>(jobs);
}

void launch_knob_stats(const KnobJob &j, void *stream) {
    // each of the three sums split over blocks of 8 warps, about 64 units per block
    const int chunks = std::max(1, std::min(1024, std::max(j.M, std::max(j.N, j.K)) / 64));
    cudaMemsetAsync(j.out, 0, sizeof(KnobStats), static_cast<cudaStream_t>(stream));
    k_knob_stats<<<3 * chunks, 256, 0, static_cast<cudaStream_t>(stream)>>>(j);
}

void launch_rowmax(const double *A, long lda, int M, int K, int32_t *er, double *ss, void *stream) {
    const int threads = 256;
    const int blocks = (M * 32 + threads - 1) / threads;
    k_rowmax<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(A, lda, M, K, er, ss);
}

void launch_colmax(const double *B, long ldb, int K, int N, int32_t *ec, double *ss, void *stream) {
    const int threads = 256;
    const int rows = 64;
    dim3 grid((N + threads - 1) / threads, (K + rows - 1) / rows);
    k_colmax<<<grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(B, ldb, K, N, rows, ec, ss);
}

void launch_split_a(const double *A, long lda, int M, int K, const int32_t *er, int b, int s, int KC, int n_kc,
                    int Mp, uint16_t *tiles, void *stream, bool trans, bool f8) {
    const int Kp = n_kc * KC;
    dim3 grid((Kp / 8 + 31) / 32, Mp / 8);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
#define OZ_CALL_A(BB) k_split_a<BB, false><<<grid, 256, 0, st>>>(A, lda, M, K, er, s, KC, n_kc, Mp, tiles, trans ? 1 : 0)
#define OZ_CALL_A8(BB) k_split_a<BB, true><<<grid, 256, 0, st>>>(A, lda, M, K, er, s, KC, n_kc, Mp, tiles, trans ? 1 : 0)
    if (f8) {
        OZ_SPLIT_DISPATCH_F8(b, OZ_CALL_A8)
    } else {
        OZ_SPLIT_DISPATCH(b, OZ_CALL_A)
    }
#undef OZ_CALL_A
#undef OZ_CALL_A8
}

void launch_split_b(const double *B, long ldb, int K, int N, const int32_t *ec, int b, int s, int KC, int n_kc,
                    int BN, int Np, uint16_t *tiles, void *stream, bool trans, bool f8) {
    const int Kp = n_kc * KC;
    dim3 grid((Np + 31) / 32, (Kp / 8 + 7) / 8);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
#define OZ_CALL_B(BB) \
    k_split_b<BB, false><<<grid, 256, 0, st>>>(B, ldb, K, N, ec, s, KC, n_kc, BN, Np, tiles, trans ? 1 : 0)
#define OZ_CALL_B8(BB) \
    k_split_b<BB, true><<<grid, 256, 0, st>>>(B, ldb, K, N, ec, s, KC, n_kc, BN, Np, tiles, trans ? 1 : 0)
    if (f8) {
        OZ_SPLIT_DISPATCH_F8(b, OZ_CALL_B8)
    } else {
        OZ_SPLIT_DISPATCH(b, OZ_CALL_B)
    }
#undef OZ_CALL_B
#undef OZ_CALL_B8
}

int launch_selftest_timeout(int *err, unsigned long long timeout_ns, void *stream) {
    k_selftest_timeout<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(err, timeout_ns);
    return 0;
}

}  // namespace ozgb
