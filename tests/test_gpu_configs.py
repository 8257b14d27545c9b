"""The measured workloads at their full sizes, held bit for bit to the oracle on
sampled rows.

* Square: M = N = K = 4096, a_ij = (U(0,1) - 0.5) exp(phi N(0,1)) with phi in
  {0.5, 1, 2, 4}, A seed 1 and B seed 2; both pair sets (fast: the triangular
  set p + q <= s - 1; accurate: the full set) for s in {3, 5, 8} slices of 7 bits.
* Long K: M = N = 8192, K = 65536, phi = 1 (operands drawn on the device), and
  the ill-conditioned variant with row i of A scaled by 2^(-40 i / M); the
  accurate configuration (s = 8, full set) and the precision knob at 1e-15.

The oracle runs the whole pipeline (row exponents over all of K, column
exponents over all of K, split, exact bins, one rounding) for the sampled rows
of A against all of B, so every bit of those rows is checked: the exponent
passes, the split, the K-blocked exact accumulation across many drains and the
epilogue.  Row exponents depend on the row alone, so the oracle needs only the
sampled rows of A (and all of B).
"""
import functools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SQ = 4096


@functools.lru_cache(maxsize=2)
def _square_inputs(phi):
    from oracle import ozoracle as O
    return O.gen_phi((SQ, SQ), 1, phi), O.gen_phi((SQ, SQ), 2, phi)


def _device_dgemm(ozlib, dA, dB, dC, s=None, J=None, bound=None):
    import torch
    M, K = dA.shape
    N = dB.shape[1]
    h = ozlib.Handle()
    if s:
        h.set_slices(s)
        h.set_bins(J or s)
    if bound:
        h.set_error_bound(bound)
    rc = h.dgemm_device(M, N, K, dA.data_ptr(), dA.stride(0), dB.data_ptr(), dB.stride(0), dC.data_ptr(),
                        dC.stride(0), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, h.last_error()
    assert h.sync() == 0, h.last_error()
    cfg = h.config()
    h.close()
    return cfg


@pytest.mark.parametrize("phi", [0.5, 1.0, 2.0, 4.0])
def test_square_4096_rows_bit_exact(ozlib, oracle, phi):
    import torch
    dev = torch.device("cuda", 0)
    A, B = _square_inputs(phi)
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    dC = torch.empty((SQ, SQ), dtype=torch.float64, device=dev)
    rows = np.array(sorted(set(oracle.sample_indices(SQ, SQ, 2, int(phi * 10))[0].tolist()) | {SQ - 1}))
    Ar = np.ascontiguousarray(A[rows])
    for s in (3, 5, 8):
        for J in (s, 2 * s - 1):
            dC.fill_(float("nan"))
            cfg = _device_dgemm(ozlib, dA, dB, dC, s, J)
            assert (cfg["slices"], cfg["bins"]) == (s, J)
            got = dC[torch.from_numpy(rows).to(dev)].cpu().numpy()
            ref = oracle.dgemm_rows(Ar, B, 7, s, J, 0, 0, len(rows))
            bad = np.flatnonzero(got.view(np.uint64) != ref.view(np.uint64))
            assert bad.size == 0, (phi, s, J, bad[:8])


def _device_phi(shape, seed, phi, dev):
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    x = torch.rand(shape, generator=g, dtype=torch.float64, device=dev).sub_(0.5)
    x.mul_(torch.randn(shape, generator=g, dtype=torch.float64, device=dev).mul_(phi).exp_())
    return x


@pytest.mark.parametrize("variant", ["phi1", "ill_conditioned"])
def test_long_k_8192x8192x65536_rows_bit_exact(ozlib, oracle, variant):
    import torch
    dev = torch.device("cuda", 0)
    M = N = 8192
    K = 65536
    dA = _device_phi((M, K), 31, 1.0, dev)
    if variant == "ill_conditioned":
        dA.mul_(torch.exp2(-40.0 * torch.arange(M, dtype=torch.float64, device=dev) / M)[:, None])
    dB = _device_phi((K, N), 32, 1.0, dev)
    dC = torch.empty((M, N), dtype=torch.float64, device=dev)
    rows = np.array([0, 2777, M - 1])
    ri = torch.from_numpy(rows).to(dev)
    Ar = dA.index_select(0, ri).cpu().numpy()
    Bh = dB.cpu().numpy()
    for label, s, J, bound in (("accurate", 8, 15, None), ("adaptive", None, None, 1e-15)):
        dC.fill_(float("nan"))
        cfg = _device_dgemm(ozlib, dA, dB, dC, s, J, bound)
        assert cfg["k_chunk"] * cfg["drain_chunks"] < K  # many drains per tile
        got = dC.index_select(0, ri).cpu().numpy()
        ref = oracle.dgemm_rows(Ar, Bh, 7, cfg["slices"], cfg["bins"], 0, 0, len(rows))
        bad = np.flatnonzero(got.view(np.uint64) != ref.view(np.uint64))
        assert bad.size == 0, (variant, label, cfg["slices"], cfg["bins"], bad[:8])
    del dA, dB, dC
    torch.cuda.empty_cache()
