/*
 * oz_oracle.c -- CPU restatement of the Oz-AIE Ozaki-scheme arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See oz_oracle.h for the parity status
 * of each stage: the host decode is pinned against the reference's own compiled
 * function; the split / bins / device sum are "parity unpinned" restatements.
 *
 * Every function cites the reference lines it follows.  Paths are relative to
 * the reference project root (atlarge-research/ozAIE):
 *   include/oz_aie.h
 *   src/aie_kernels/generic/ozaki_base.cc
 *   src/aie_kernels/aie2p/mm_ozaki.cc
 *   src/programming_examples/basic/matrix_multiplication/common.h
 */
#include "oz_oracle.h"

#include <dlfcn.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
typedef __int128 i128;

static inline uint64_t dbits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double bitsd(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static inline int expfield(uint64_t u) { return (int)((u >> 52) & 0x7FF); }

int ozo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 0;
#endif
}

/* ---------------------------------------------------------------- stage (a) */
/* ozaki_base.cc:403-426: exponent = (hi_word << 1) >> 21, i.e. bits 52..62 of the
 * double; *ps = max(*ps, reduce_max(group)) with the buffer zeroed first
 * (ozaki_base.cc:820-825, whole_array_iron_ozaki.py:470-483), over all of K. */
void ozo_max_exp_rows(const double *A, int M, int K, int32_t *Er) {
    for (int m = 0; m < M; ++m) {
        int e = 0;
        const double *row = A + (long)m * K;
        for (int k = 0; k < K; ++k) {
            int f = expfield(dbits(row[k]));
            if (f > e) e = f;
        }
        Er[m] = e;
    }
}

void ozo_max_exp_cols(const double *B, int K, int N, int32_t *Ec) {
    for (int n = 0; n < N; ++n) Ec[n] = 0;
    for (int k = 0; k < K; ++k) {
        const double *row = B + (long)k * N;
        for (int n = 0; n < N; ++n) {
            int f = expfield(dbits(row[n]));
            if (f > Ec[n]) Ec[n] = f;
        }
    }
}

/* ---------------------------------------------------------------- stage (b) */
/* extract_splits_acc64_half_half, ozaki_base.cc:449-639.
 *  - bits_to_avoid = 1 + (b == 3 ? 3 : 0)                          (:459)
 *  - valid bits nv0 = 64 - avoid - ((64 - avoid) % b)               (:461-464)
 *  - one 64-bit window when d*b <= nv0, else two                    (:465)
 *  - sign from the high word, exponent bias = E - e as uint32       (:497-509)
 *  - implicit one only for normal numbers (subnormals keep bias E-0)(:507,:516)
 *  - the 53-bit mantissa is aligned to bit 63 of the high word      (:520-527)
 *  - four 32-bit words selected by bias >= 32/64/96; the fourth word is NOT
 *    cleared for bias >= 128 (quirk kept)                           (:534-545)
 *  - remaining shift r = bias mod 32 applied to the word stream      (:551-576)
 *  - slices are the next b bits from the top, truncated, sign applied(:609-628)
 * Restated: X = (w0:w1:w2:w3) >> r as a 128-bit number and
 *   slice_i = sign * ((X >> (128 - b(i+1))) & (2^b - 1)).
 * With one window only (w2 = w3 = 0) the same formula holds because every slice
 * lies in the top nv0 <= 63 bits. */
void ozo_split_elem(uint64_t x, int E, int b, int d, int8_t *out, long stride) {
    const int avoid = 1 + (b == 3 ? 3 : 0);
    const int nv0 = 64 - avoid - ((64 - avoid) % b);
    const int nacc = (d * b <= nv0) ? 1 : 2;
    const int sign = (int)(x >> 63);
    const uint32_t e = (uint32_t)expfield(x);
    const uint64_t mant = (x & ((1ULL << 52) - 1)) | (e ? (1ULL << 52) : 0);
    const uint32_t bias = (uint32_t)E - e;
    const uint64_t m64 = mant << 11;
    const uint32_t vhi = (uint32_t)(m64 >> 32), vlo = (uint32_t)m64;
    uint32_t w0 = bias >= 32u ? 0u : vhi;
    uint32_t w1 = bias >= 64u ? 0u : (bias >= 32u ? vhi : vlo);
    uint32_t w2 = 0, w3 = 0;
    if (nacc == 2) {
        w2 = bias >= 96u ? 0u : (bias >= 64u ? vhi : (bias >= 32u ? vlo : 0u));
        w3 = bias >= 96u ? vhi : (bias >= 64u ? vlo : 0u);
    }
    const unsigned r = bias & 31u;
    const u128 W = ((u128)(((uint64_t)w0 << 32) | w1) << 64) | (u128)(((uint64_t)w2 << 32) | w3);
    const u128 X = W >> r;
    const unsigned mask = (1u << b) - 1u;
    for (int i = 0; i < d; ++i) {
        int sh = 128 - b * (i + 1);
        int v = (sh >= 0) ? (int)((unsigned)(X >> sh) & mask) : 0;
        out[(long)i * stride] = (int8_t)(sign ? -v : v);
    }
}

void ozo_split_rows(const double *A, int M, int K, const int32_t *Er, int b, int d, int8_t *planes) {
    const long plane = (long)M * K;
#pragma omp parallel for schedule(static)
    for (int m = 0; m < M; ++m)
        for (int k = 0; k < K; ++k)
            ozo_split_elem(dbits(A[(long)m * K + k]), Er[m], b, d, planes + (long)m * K + k, plane);
}

void ozo_split_cols(const double *B, int K, int N, const int32_t *Ec, int b, int d, int8_t *planes) {
    const long plane = (long)K * N;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < K; ++k)
        for (int n = 0; n < N; ++n)
            ozo_split_elem(dbits(B[(long)k * N + n]), Ec[n], b, d, planes + (long)k * N + n, plane);
}

/* ---------------------------------------------------------------- stage (c) */
/* ozaki_matmul, aie2p/mm_ozaki.cc:255-308: for a in 0..d-1, for b in 0..d-1-a,
 * bins[a+b] += A_a . B_b (int8 x int8 -> int32 micro-GEMMs, upstream
 * matmul_vectorized_8x8x8_i8_i32).  Here the sums are kept exactly in int64; the
 * pair set is {p + q <= J - 1, p < d, q < d}, J = d being the reference's. */
void ozo_bins(const int8_t *Ap, const int8_t *Bp, int M, int N, int K, int d, int J, int64_t *bins) {
    const long aplane = (long)M * K, bplane = (long)K * N, cplane = (long)M * N;
    const int KBLK = 2048; /* int32 partial sums stay below 2^31 for <= 64 pairs */
#pragma omp parallel
    {
        int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
        int64_t *acc = (int64_t *)malloc(sizeof(int64_t) * (size_t)N);
#pragma omp for schedule(dynamic, 1)
        for (int m = 0; m < M; ++m) {
            for (int j = 0; j < J; ++j) {
                for (int n = 0; n < N; ++n) acc[n] = 0;
                int plo = j - (d - 1) > 0 ? j - (d - 1) : 0;
                int phi = j < d - 1 ? j : d - 1;
                for (int k0 = 0; k0 < K; k0 += KBLK) {
                    int k1 = k0 + KBLK < K ? k0 + KBLK : K;
                    for (int n = 0; n < N; ++n) tmp[n] = 0;
                    for (int p = plo; p <= phi; ++p) {
                        int q = j - p;
                        const int8_t *arow = Ap + p * aplane + (long)m * K;
                        const int8_t *bq = Bp + q * bplane;
                        for (int k = k0; k < k1; ++k) {
                            int32_t a = arow[k];
                            if (!a) continue;
                            const int8_t *brow = bq + (long)k * N;
                            for (int n = 0; n < N; ++n) tmp[n] += a * (int32_t)brow[n];
                        }
                    }
                    for (int n = 0; n < N; ++n) acc[n] += tmp[n];
                }
                int64_t *out = bins + j * cplane + (long)m * N;
                for (int n = 0; n < N; ++n) out[n] = acc[n];
            }
        }
        free(tmp);
        free(acc);
    }
}

/* ---------------------------------------------------------------- stage (d) */
/* n_bins_in_first_group, ozaki_base.cc:151-158 (host copy include/oz_aie.h:98-103);
 * log2K is countr_zero(K) exactly as the reference computes it. */
int ozo_first_group(int K, int b, int d) {
    int ctz = K ? __builtin_ctz((unsigned)K) : 32;
    int alignable = 31 / b + 1;
    int numer = b * (d + 1) - 51 + ctz;
    int minfirst = numer < 0 ? 1 : (numer / b + 1);
    int g0 = minfirst > alignable ? minfirst : alignable;
    return g0 < d ? g0 : d;
}

/* ozaki_vectorized_sum_upshift, ozaki_base.cc:279-328: the bins are int32
 * (aie::accum<acc64>.from_vector(int32, b*i) sign-extends and shifts); group 0
 * sums bins d-1, d-2, ... g0 of them, group 1 the rest, each with weight 2^{b t};
 * bits 51..62 of hi are replaced by Er + Ec and bit 63 kept (:293-317). */
void ozo_sum_upshift(const int64_t *bins, const int32_t *Er, const int32_t *Ec, int M, int N, int K,
                     int b, int d, int64_t *pairs) {
    const int g0 = ozo_first_group(K, b, d), g1 = d - g0;
    const long cplane = (long)M * N;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long idx = (long)m * N + n;
            uint64_t lo = 0, hi = 0;
            for (int t = 0; t < g0; ++t)
                lo += (uint64_t)(int64_t)(int32_t)(uint32_t)bins[(d - 1 - t) * cplane + idx] << (b * t);
            for (int t = 0; t < g1; ++t)
                hi += (uint64_t)(int64_t)(int32_t)(uint32_t)bins[(d - 1 - g0 - t) * cplane + idx] << (b * t);
            uint64_t scale = (uint64_t)(uint32_t)(Er[m] + Ec[n]);
            hi = (hi & 0x8007FFFFFFFFFFFFULL) | ((scale & 0xFFFULL) << 51);
            pairs[2 * idx] = (int64_t)lo;
            pairs[2 * idx + 1] = (int64_t)hi;
        }
}

static inline int clz128(u128 v) {
    uint64_t h = (uint64_t)(v >> 64), l = (uint64_t)v;
    if (h) return __builtin_clzll(h);
    if (l) return 64 + __builtin_clzll(l);
    return 128;
}

/* The reference's bit arithmetic (include/oz_aie.h:124-146) applied to a signed
 * 128-bit magnitude source quad with scale Er+Ec and exponent offset b(d+1):
 *   lz over 128 bits, exponent = (128 - lz) - b(d+1) - 1, truncate to 53 bits,
 *   lu = mant - 2^52 + sign + (exponent + 1023) << 52 + (Er+Ec+2-2046) << 52,
 *   all modulo 2^64; quad == 0 gives +0.0. */
static double ref_decode_quad(i128 quad, int64_t escale, int bd1) {
    i128 quad_sign = quad & ((i128)1 << 127);
    if (quad_sign) quad = -quad;
    int lz = clz128((u128)quad);
    int64_t exponent = (int64_t)(128 - lz) - bd1 - 1;
    int shift = (128 - lz) - 53;
    uint64_t lu = shift > 0 ? (uint64_t)((u128)quad >> shift) : (uint64_t)((u128)quad << -shift);
    if (lu > 0) {
        uint64_t scale_back = (uint64_t)(escale + 2 - 2046) << 52;
        lu -= 0x0010000000000000ULL;
        lu += (quad_sign ? 0x8000000000000000ULL : 0ULL) + ((uint64_t)(exponent + 1023) << 52) + scale_back;
    }
    return bitsd(lu);
}

/* convert_paired_i64_to_double_matrix, include/oz_aie.h:92-150. */
void ozo_decode_pairs(const int64_t *pairs, double *C, int M, int N, int K, int d, int b) {
    const int g0 = ozo_first_group(K, b, d);
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long idx = (long)m * N + n;
            int64_t lo = pairs[2 * idx], hi = pairs[2 * idx + 1];
            /* hi bits 51..62 hold Er+Ec; bit 63 is the sign of the hi group sum */
            int64_t escale = (int64_t)(((uint64_t)hi >> 51) & 0xFFF);
            uint64_t hmag = (uint64_t)hi & 0x0007FFFFFFFFFFFFULL;
            int64_t hsig = (hi < 0) ? (int64_t)(hmag | 0xFFF8000000000000ULL) : (int64_t)hmag;
            i128 quad = (i128)lo + ((i128)hsig << (g0 * b));
            C[idx] = ref_decode_quad(quad, escale, b * (d + 1));
        }
}

/* ------------------------------------------------ exact big-integer rounding */
/* A little-endian array of 32-bit words holding a non-negative magnitude. */
static int bitlen_words(const uint32_t *w, int n) {
    for (int i = n - 1; i >= 0; --i)
        if (w[i]) return 32 * i + (32 - __builtin_clz(w[i]));
    return 0;
}
static inline int get_bit(const uint32_t *w, int n, long i) {
    if (i < 0 || i >= 32L * n) return 0;
    return (int)((w[i >> 5] >> (i & 31)) & 1u);
}
static int any_below(const uint32_t *w, int n, long i) { /* any bit with index < i */
    if (i <= 0) return 0;
    long full = i >> 5;
    for (long k = 0; k < full && k < n; ++k)
        if (w[k]) return 1;
    if (full < n && (i & 31)) {
        uint32_t m = (1u << (i & 31)) - 1u;
        if (w[full] & m) return 1;
    }
    return 0;
}
/* floor(mag / 2^sh) for sh >= 0, or mag << -sh; result must fit 64 bits. */
static uint64_t extract64(const uint32_t *w, int n, long sh) {
    uint64_t r = 0;
    for (int bit = 63; bit >= 0; --bit) r = (r << 1) | (uint64_t)get_bit(w, n, sh + bit);
    return r;
}

/* Correctly rounded (RN-even) or truncated double of (-1)^sign * mag * 2^e2. */
static double round_words(const uint32_t *w, int n, int sign, long e2, int rz) {
    int L = bitlen_words(w, n);
    if (L == 0) return sign ? -0.0 : 0.0;
    long elead = (long)L - 1 + e2;
    long biased = elead + 1023;
    long sh = (biased >= 1) ? (long)L - 53 : (long)L - 53 + (1 - biased);
    uint64_t m = extract64(w, n, sh);
    if (!rz) {
        int rb = get_bit(w, n, sh - 1);
        int st = any_below(w, n, sh - 1);
        if (rb && (st || (m & 1))) m++;
    }
    uint64_t bits;
    if (biased >= 1) {
        if (biased >= 2047) bits = 0x7FF0000000000000ULL;
        else {
            bits = ((uint64_t)(biased - 1) << 52) + m;
            if (bits >= 0x7FF0000000000000ULL) bits = rz ? 0x7FEFFFFFFFFFFFFFULL : 0x7FF0000000000000ULL;
        }
    } else {
        bits = m;
    }
    if (sign) bits |= 0x8000000000000000ULL;
    return bitsd(bits);
}

/* -------------------------------------------- GB300 finishing rule (oracle) */
/* q = sum_j bins_j 2^{b(J-1-j)} in 256-bit two's complement. */
static void q_accumulate(const int64_t *bins, long cplane, long idx, int b, int J, uint64_t q[4]) {
    q[0] = q[1] = q[2] = q[3] = 0;
    for (int j = 0; j < J; ++j) {
        int64_t v = bins[j * cplane + idx];
        int sh = b * (J - 1 - j);
        uint64_t ext = v < 0 ? ~0ULL : 0ULL;
        uint64_t t[4] = {(uint64_t)v, ext, ext, ext};
        /* shift the 256-bit t left by sh */
        int ws = sh >> 6, bs = sh & 63;
        uint64_t s[4] = {0, 0, 0, 0};
        for (int i = 3; i >= 0; --i) {
            int src = i - ws;
            if (src < 0) continue;
            uint64_t lo = t[src] << bs;
            uint64_t carry = (bs && src - 1 >= 0) ? (t[src - 1] >> (64 - bs)) : 0;
            s[i] = lo | carry;
        }
        unsigned __int128 c = 0;
        for (int i = 0; i < 4; ++i) {
            c += (unsigned __int128)q[i] + s[i];
            q[i] = (uint64_t)c;
            c >>= 64;
        }
    }
}

void ozo_finish(const int64_t *bins, const int32_t *Er, const int32_t *Ec, int M, int N, int b, int J,
                int rounding, double *C, int64_t *q_out) {
    const long cplane = (long)M * N;
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            long idx = (long)m * N + n;
            uint64_t q[4];
            q_accumulate(bins, cplane, idx, b, J, q);
            if (q_out)
                for (int i = 0; i < 4; ++i) q_out[4 * idx + i] = (int64_t)q[i];
            int sign = (int)(q[3] >> 63);
            uint64_t mag[4];
            if (sign) {
                unsigned __int128 c = 1;
                for (int i = 0; i < 4; ++i) {
                    c += (unsigned __int128)(~q[i]);
                    mag[i] = (uint64_t)c;
                    c >>= 64;
                }
            } else {
                memcpy(mag, q, sizeof mag);
            }
            if (rounding == 1) {
                /* reference arithmetic on the (at most 128-bit) magnitude */
                i128 quad = (i128)(((u128)mag[1] << 64) | mag[0]);
                if (sign) quad = -quad;
                C[idx] = ref_decode_quad(quad, (int64_t)Er[m] + Ec[n], b * (J + 1));
            } else {
                uint32_t w[8];
                for (int i = 0; i < 4; ++i) {
                    w[2 * i] = (uint32_t)mag[i];
                    w[2 * i + 1] = (uint32_t)(mag[i] >> 32);
                }
                long e2 = (long)Er[m] + Ec[n] - 2044 - (long)b * (J + 1);
                C[idx] = round_words(w, 8, sign, e2, 0);
            }
        }
}

void ozo_dgemm_rows(const double *A, const double *B, double *C, int M, int N, int K, int b, int d,
                    int J, int rounding, int r0, int r1) {
    int R = r1 - r0;
    int32_t *Er = (int32_t *)malloc(sizeof(int32_t) * (size_t)R);
    int32_t *Ec = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    int8_t *Ap = (int8_t *)malloc((size_t)d * R * K);
    int8_t *Bp = (int8_t *)malloc((size_t)d * K * N);
    int64_t *bins = (int64_t *)malloc(sizeof(int64_t) * (size_t)J * R * N);
    const double *Ar = A + (long)r0 * K;
    ozo_max_exp_rows(Ar, R, K, Er);
    ozo_max_exp_cols(B, K, N, Ec);
    ozo_split_rows(Ar, R, K, Er, b, d, Ap);
    ozo_split_cols(B, K, N, Ec, b, d, Bp);
    ozo_bins(Ap, Bp, R, N, K, d, J, bins);
    ozo_finish(bins, Er, Ec, R, N, b, J, rounding, C + (long)r0 * N, NULL);
    free(Er); free(Ec); free(Ap); free(Bp); free(bins);
    (void)M;
}

void ozo_dgemm(const double *A, const double *B, double *C, int M, int N, int K, int b, int d, int J,
               int rounding) {
    ozo_dgemm_rows(A, B, C, M, N, K, b, d, J, rounding, 0, M);
}

/* ------------------------------------------------------ exact dot products */
/* Kulisch-style accumulator: 32-bit digits in int64 limbs (carry-save), bit 0 at
 * weight 2^-2200, enough for every product of two finite doubles. */
#define KUL_OFF 2200
#define KUL_LIMBS 142
static void kul_add(int64_t *acc, double a, double b) {
    uint64_t ua = dbits(a), ub = dbits(b);
    int ea = expfield(ua), eb = expfield(ub);
    if (ea == 2047 || eb == 2047) return; /* inf / nan: not supported by the exact oracle */
    uint64_t ma = (ua & ((1ULL << 52) - 1)) | (ea ? (1ULL << 52) : 0);
    uint64_t mb = (ub & ((1ULL << 52) - 1)) | (eb ? (1ULL << 52) : 0);
    if (!ma || !mb) return;
    int sa = (int)(ua >> 63) ^ (int)(ub >> 63);
    long e2 = (long)(ea ? ea : 1) - 1075 + (long)(eb ? eb : 1) - 1075;
    long pos = e2 + KUL_OFF;
    u128 p = (u128)ma * mb;
    int li = (int)(pos >> 5), sh = (int)(pos & 31);
    /* p << sh spans at most 138 bits -> 5 digits */
    uint32_t dg[5];
    u128 lo = p << sh;
    uint64_t top = sh ? (uint64_t)(p >> (128 - sh)) : 0;
    dg[0] = (uint32_t)lo; dg[1] = (uint32_t)(lo >> 32); dg[2] = (uint32_t)(lo >> 64);
    dg[3] = (uint32_t)(lo >> 96); dg[4] = (uint32_t)top;
    for (int i = 0; i < 5; ++i) {
        if (sa) acc[li + i] -= dg[i];
        else acc[li + i] += dg[i];
    }
}
static double kul_round(int64_t *acc) {
    /* normalise to two's complement 32-bit digits */
    for (int i = 0; i < KUL_LIMBS - 1; ++i) {
        int64_t c = acc[i] >> 32; /* arithmetic */
        acc[i] -= c * 4294967296LL;
        acc[i + 1] += c;
    }
    int sign = acc[KUL_LIMBS - 1] < 0;
    uint32_t w[KUL_LIMBS];
    if (sign) {
        /* magnitude = -(value): negate the digit vector */
        int64_t borrow = 0;
        for (int i = 0; i < KUL_LIMBS; ++i) {
            int64_t v = -acc[i] - borrow;
            borrow = 0;
            while (v < 0) { v += 4294967296LL; borrow++; }
            w[i] = (uint32_t)v;
        }
    } else {
        for (int i = 0; i < KUL_LIMBS; ++i) w[i] = (uint32_t)acc[i];
    }
    return round_words(w, KUL_LIMBS, sign, -KUL_OFF, 0);
}

void ozo_exact_entries(const double *A, const double *B, int M, int N, int K, const int32_t *rows,
                       const int32_t *cols, int n, double *out, double *absdot) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < n; ++i) {
        int64_t acc[KUL_LIMBS];
        memset(acc, 0, sizeof acc);
        double s = 0.0;
        int r = rows[i], c = cols[i];
        for (int k = 0; k < K; ++k) {
            double a = A[(long)r * K + k], b = B[(long)k * N + c];
            kul_add(acc, a, b);
            s += fabs(a) * fabs(b);
        }
        out[i] = kul_round(acc);
        if (absdot) absdot[i] = s;
    }
    (void)M;
}

/* ------------------------------------------------------------------ MPFR */
/* Layout of mpfr_t on LP64 targets (mpfr.h of MPFR 4.x): {prec, sign, exp, limbs}. */
typedef struct { long prec; int sign; long exp; void *d; } ozo_mpfr_rec;
typedef void (*mpfr_init2_fn)(ozo_mpfr_rec *, long);
typedef int (*mpfr_set_d_fn)(ozo_mpfr_rec *, double, int);
typedef int (*mpfr_binop_fn)(ozo_mpfr_rec *, const ozo_mpfr_rec *, const ozo_mpfr_rec *, int);
typedef double (*mpfr_get_d_fn)(const ozo_mpfr_rec *, int);
typedef void (*mpfr_clear_fn)(ozo_mpfr_rec *);

int ozo_mpfr_entries(const double *A, const double *B, int M, int N, int K, const int32_t *rows,
                     const int32_t *cols, int n, int prec, double *out) {
    static void *h = NULL;
    if (!h) h = dlopen("libmpfr.so.6", RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    mpfr_init2_fn init2 = (mpfr_init2_fn)dlsym(h, "mpfr_init2");
    mpfr_set_d_fn set_d = (mpfr_set_d_fn)dlsym(h, "mpfr_set_d");
    mpfr_binop_fn mul = (mpfr_binop_fn)dlsym(h, "mpfr_mul");
    mpfr_binop_fn add = (mpfr_binop_fn)dlsym(h, "mpfr_add");
    mpfr_get_d_fn get_d = (mpfr_get_d_fn)dlsym(h, "mpfr_get_d");
    mpfr_clear_fn clear = (mpfr_clear_fn)dlsym(h, "mpfr_clear");
    if (!init2 || !set_d || !mul || !add || !get_d || !clear) return -1;
    const int RNDN = 0;
    /* common.h:211-232: elem_a, elem_b, prod, running_sum at prec bits, RNDN */
    for (int i = 0; i < n; ++i) {
        ozo_mpfr_rec ea, eb, prod, sum;
        init2(&ea, prec); init2(&eb, prec); init2(&prod, prec); init2(&sum, prec);
        set_d(&sum, 0.0, RNDN);
        int r = rows[i], c = cols[i];
        for (int k = 0; k < K; ++k) {
            set_d(&ea, A[(long)r * K + k], RNDN);
            set_d(&eb, B[(long)k * N + c], RNDN);
            mul(&prod, &ea, &eb, RNDN);
            add(&sum, &sum, &prod, RNDN);
        }
        out[i] = get_d(&sum, RNDN);
        clear(&ea); clear(&eb); clear(&prod); clear(&sum);
    }
    (void)M;
    return 0;
}

/* matmul_DGEMM, common.h:234-254 (row-major B, row-major C). */
void ozo_dgemm_naive(const double *A, const double *B, double *C, int M, int N, int K) {
    for (int m = 0; m < M; ++m)
        for (int n = 0; n < N; ++n) {
            double s = 0.0;
            for (int k = 0; k < K; ++k) s += A[(long)m * K + k] * B[(long)k * N + n];
            C[(long)m * N + n] = s;
        }
}
