"""One DGEMM sharded over ranks (ozaie_gb300.sharded): the partition, the gather
and the bit-identity of the gathered product with the single-rank product.

On CPU the ranks are gloo processes whose local block product is the oracle's
pipeline (the stand-in for a GPU that this machine lacks); the partition and
the gather under test are the library's.  On the GPU machine two ranks share the
one GPU, each with its own handle: their kernels never wait on each other (the
path has no device-side exchange), so this exercises the GPU block product and
the host gather together.
"""
import os
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import HAVE_GPU, ROOT


def test_grid_covers_c_once():
    from ozaie_gb300 import sharded
    for world in (1, 2, 3, 4, 6, 8):
        for M, N in ((256, 256), (1000, 300), (64, 4096), (8, 8)):
            pr, pc = sharded.grid_shape(world, M, N)
            assert pr * pc == world
            seen = np.zeros((M, N), np.int32)
            for r in range(world):
                r0, r1, c0, c1 = sharded.block_range(r, world, M, N)
                assert r1 > r0 and c1 > c0
                seen[r0:r1, c0:c1] += 1
            assert (seen == 1).all()
    assert sharded.grid_shape(4, 4096, 4096) == (2, 2)
    assert sharded.grid_shape(2, 8192, 512) == (2, 1)
    with pytest.raises(ValueError):
        sharded.block_range(4, 4, 64, 64)


def _oracle_local(b, s, J):
    from oracle import ozoracle as O

    def run(A_rows, B_cols):
        # the block's own exponents: rows of A and columns of B over all of K
        return O.dgemm(A_rows, B_cols, b, s, J, 0)
    return run


def _worker(rank, world, port, out, use_gpu):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from ozaie_gb300 import sharded
    from oracle import ozoracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        M, N, K = 300, 200, 700
        A = O.gen_phi((M, K), 81, 1.0)
        B = O.gen_phi((K, N), 82, 1.0)
        if use_gpu:
            import torch
            import ozaie_gb300 as oz
            torch.cuda.set_device(0)
            h = oz.Handle()
            h.set_slices(9)
            h.set_bins(9)
            local = sharded.gpu_block_dgemm(h, oz.Mode.fast)
        else:
            local = _oracle_local(7, 9, 9)
        C, rng = sharded.dgemm_sharded(A, B, local)
        blk, rng2 = sharded.dgemm_sharded(A, B, local, gather=False)
        assert rng == rng2
        if use_gpu:
            h.close()
        out.put((rank, rng, None if C is None else C.tobytes(), blk.tobytes()))
    finally:
        dist.barrier()
        dist.destroy_process_group()


def _run(world, use_gpu):
    from oracle import ozoracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 31500 + (os.getpid() * 7 + world) % 1000
    ps = [ctx.Process(target=_worker, args=(r, world, port, q, use_gpu)) for r in range(world)]
    for p in ps:
        p.start()
    res = {}
    for _ in range(world):
        rank, rng, C, blk = q.get(timeout=300)
        res[rank] = (rng, C, blk)
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    M, N, K = 300, 200, 700
    A = O.gen_phi((M, K), 81, 1.0)
    B = O.gen_phi((K, N), 82, 1.0)
    ref = O.dgemm(A, B, 7, 9, 9, 0)
    C = np.frombuffer(res[0][1], np.float64).reshape(M, N)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))
    for r in range(1, world):
        assert res[r][1] is None
    for r in range(world):
        r0, r1, c0, c1 = res[r][0]
        blk = np.frombuffer(res[r][2], np.float64).reshape(r1 - r0, c1 - c0)
        assert np.array_equal(blk.view(np.uint64), ref[r0:r1, c0:c1].view(np.uint64))


@pytest.mark.parametrize("world", [2, 4])
def test_sharded_gloo_matches_single_rank_bits(world):
    _run(world, use_gpu=False)


@pytest.mark.gpu
def test_sharded_two_ranks_on_the_gpu():
    if not HAVE_GPU:
        pytest.skip("no GPU")
    _run(2, use_gpu=True)
