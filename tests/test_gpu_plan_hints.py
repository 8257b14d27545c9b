"""Slice-pair GEMM plans forced through ozgb_set_plan_hint, held bit for bit to
the oracle: one, two and three issuing warps (the UMMA runs of a K step dealt
round-robin), bin-block partitions other than the planner's, and double-buffered
blocks (a second TMEM accumulator range per block, switched at each drain).
K = 1100 gives every block several drains per tile; M and N are not multiples of
the tile."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M, N, K = 300, 200, 1100
ROWS = np.array([0, 1, 127, 128, 255, 299])

CASES = [
    (8, 9, {}),
    (8, 9, dict(issuers=1)),
    (8, 9, dict(issuers=2)),
    (8, 9, dict(tile_n=48, block_nb=(2, 3, 4))),
    (8, 9, dict(tile_n=48, block_nb=(4, 5), issuers=2)),
    (8, 9, dict(tile_n=32, block_nb=(4, 5), dbl=1)),
    (8, 9, dict(tile_n=32, block_nb=(2, 2, 2, 3), dbl=1)),
    (5, 6, dict(dbl=1)),
    (11, 12, dict(dbl=1, issuers=3)),
    (8, 15, dict(tile_n=32, k_chunk=16)),
]


@pytest.fixture(scope="module")
def operands():
    from oracle import ozoracle as O
    return O.gen_phi((M, K), 61, 1.0), O.gen_phi((K, N), 62, 1.0)


@pytest.mark.parametrize("s,J,hint", CASES)
def test_plan_hint_bit_exact(ozlib, oracle, operands, s, J, hint):
    import torch
    A, B = operands
    dev = torch.device("cuda", 0)
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    dC = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
    h = ozlib.Handle()
    h.set_slices(s)
    h.set_bins(J)
    if hint:
        h.set_plan_hint(**hint)
    rc = h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N,
                        torch.cuda.current_stream().cuda_stream)
    assert rc == 0, h.last_error()
    assert h.sync() == 0, h.last_error()
    cfg = h.config()
    h.close()
    if "issuers" in hint:
        assert cfg["issuers"] == hint["issuers"]
    if "block_nb" in hint:
        assert cfg["block_nb"][:cfg["blocks"]] == list(hint["block_nb"])
    if hint.get("dbl") == 1 and hint.get("tile_n") == 32:
        assert cfg["dbl_blocks"] != 0
    got = dC.cpu().numpy()[ROWS]
    ref = oracle.dgemm_rows(np.ascontiguousarray(A[ROWS]), B, 7, s, J, 0, 0, len(ROWS))
    bad = np.flatnonzero(got.view(np.uint64) != ref.view(np.uint64))
    assert bad.size == 0, (s, J, hint, cfg, bad[:8])


def test_plan_hint_that_cannot_hold_fails(ozlib):
    import torch
    dev = torch.device("cuda", 0)
    dA = torch.zeros((64, 64), dtype=torch.float64, device=dev)
    h = ozlib.Handle()
    h.set_slices(8)
    h.set_bins(9)
    h.set_plan_hint(tile_n=48, block_nb=(4, 4))  # covers 8 of the 9 bins
    rc = h.dgemm_device(64, 64, 64, dA.data_ptr(), 64, dA.data_ptr(), 64, dA.data_ptr(), 64,
                        torch.cuda.current_stream().cuda_stream)
    assert rc != 0 and "hinted bin blocks" in h.last_error()
    h.close()
