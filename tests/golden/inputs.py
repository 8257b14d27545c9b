"""Deterministic test inputs shared by the fixture generator and the tests.

`uniform64(seed, lo, hi, n)` reproduces `std::mt19937_64(seed)` followed by
`std::uniform_real_distribution<double>(lo, hi)` as libstdc++ implements it
(one 64-bit draw per value: x -> double(x) / 2^64, clamped below 1, then
lo + u * (hi - lo) evaluated as u * (hi - lo) + lo).  The generator is the
published MT19937-64 of Matsumoto and Nishimura.  The committed fixtures record
the SHA-256 of the same values produced by the C++ standard library
(gen_inputs.cpp), so a test can check that this restatement matches it.
"""
import hashlib

import numpy as np

_MASK = (1 << 64) - 1
_NN, _MM = 312, 156
_MATRIX_A = 0xB5026F5AA96619E9
_UM = _MASK ^ ((1 << 31) - 1)
_LM = (1 << 31) - 1


def mt19937_64(seed, count):
    mt = [0] * _NN
    mt[0] = seed & _MASK
    for i in range(1, _NN):
        mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & _MASK
    out = []
    idx = _NN
    while len(out) < count:
        if idx >= _NN:
            for i in range(_NN):
                x = (mt[i] & _UM) | (mt[(i + 1) % _NN] & _LM)
                xa = x >> 1
                if x & 1:
                    xa ^= _MATRIX_A
                mt[i] = mt[(i + _MM) % _NN] ^ xa
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        out.append(y & _MASK)
    return out


def uniform64(seed, lo, hi, count):
    one_below = np.nextafter(1.0, 0.0)
    vals = np.empty(count, np.float64)
    for i, x in enumerate(mt19937_64(seed, count)):
        u = float(x) / 18446744073709551616.0
        if u >= 1.0:
            u = one_below
        vals[i] = u * (hi - lo) + lo
    return vals


def uniform_256x512x128_inputs():
    """Row-major A (256 x 128) and B (128 x 512), uniform(-1, 1), one
    mt19937_64(0) stream drawn A first, then B."""
    M, N, K = 256, 512, 128
    v = uniform64(0, -1.0, 1.0, M * K + K * N)
    return v[:M * K].reshape(M, K), v[M * K:].reshape(K, N)


def sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
