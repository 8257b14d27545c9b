"""One Ozaki DGEMM sharded over the GPUs of a node: one process per GPU, no
collective in the compute path.

Partition.  The R ranks form a pr x pc grid; rank r = (i, j), i = r // pc,
j = r % pc, computes the C block of rows [M i / pr, M (i + 1) / pr) and columns
[N j / pc, N (j + 1) / pc) from those rows of A and those columns of B.  This is
the output-stationary 2D spread of C over a compute array, with A shared along
the grid's rows and B along its columns, that the reference uses across its AIE
cores (src/programming_examples/.../whole_array_iron_ozaki.py:182-227, the
A/B broadcast at :353-434).

Why no exchange is needed.  Stage (a) takes a row's exponent over all of K of
that row of A, and a column's over all of K of that column of B; stages (b)-(d)
of an entry use only its row's and column's slices.  So each rank's block is
bit-identical to the same block of the single-GPU product, with no exponent
max-reduction and no exchange of bins or partial sums.  (A split along K would
need both: a max over ranks before the split and an exact integer sum of bins
before the rounding; it is not used.)  The optional gather of the blocks onto
one rank is the only collective, after all compute.
"""
import numpy as np


def grid_shape(world, M, N):
    """(pr, pc) with pr * pc == world minimising the operand bytes each rank
    reads, K (M / pr + N / pc)."""
    best = None
    for pr in range(1, world + 1):
        if world % pr:
            continue
        pc = world // pr
        if pr > M or pc > N:
            continue
        cost = M / pr + N / pc
        if best is None or cost < best[0]:
            best = (cost, pr, pc)
    if best is None:
        raise ValueError("a %d x %d product cannot be split over %d ranks" % (M, N, world))
    return best[1], best[2]


def block_range(rank, world, M, N, grid=None):
    """Rows [r0, r1) and columns [c0, c1) of C computed by `rank`."""
    pr, pc = grid or grid_shape(world, M, N)
    if pr * pc != world or not 0 <= rank < world:
        raise ValueError("rank %d outside a %d x %d grid" % (rank, pr, pc))
    i, j = divmod(rank, pc)
    return M * i // pr, M * (i + 1) // pr, N * j // pc, N * (j + 1) // pc


def gpu_block_dgemm(handle, mode):
    """The local product of one rank on its GPU: the drop-in host-array call
    (ozAIE_setup + ozAIE_DGEMM semantics) on this rank's rows of A and columns
    of B.  `handle` is an ozaie_gb300.Handle on the rank's current device."""
    def run(A_rows, B_cols):
        m, k = A_rows.shape
        n = B_cols.shape[1]
        rc = handle.setup(m, n, k, mode)
        if rc:
            raise RuntimeError("ozgb_setup: %s" % handle.last_error())
        C = np.empty((m, n), np.float64)
        rc = handle.dgemm(m, n, k, np.ascontiguousarray(A_rows), np.ascontiguousarray(B_cols), C)
        if rc:
            raise RuntimeError("ozgb_dgemm: %s" % handle.last_error())
        return C
    return run


def dgemm_sharded(A, B, local, group=None, grid=None, gather=True, dst=0):
    """C = A B over the ranks of `group` (torch.distributed, default group).

    A (M x K) and B (K x N) are row-major float64 host arrays; each rank reads
    only its rows of A and columns of B.  `local(A_rows, B_cols)` computes one
    block (gpu_block_dgemm for the GPU path).  Returns (C, (r0, r1, c0, c1)):
    with gather, C is the whole product on rank `dst` (None elsewhere);
    without, C is this rank's block.
    """
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    M, K = A.shape
    if B.shape[0] != K:
        raise ValueError("inner dimensions differ")
    N = B.shape[1]
    grid = grid or grid_shape(world, M, N)
    r0, r1, c0, c1 = block_range(rank, world, M, N, grid)
    blk = np.ascontiguousarray(local(A[r0:r1], B[:, c0:c1]), np.float64)
    if blk.shape != (r1 - r0, c1 - c0):
        raise ValueError("local product has shape %s, expected %s" % (blk.shape, (r1 - r0, c1 - c0)))
    if not gather:
        return blk, (r0, r1, c0, c1)
    # the blocks travel as device tensors under NCCL, host tensors otherwise
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else None
    if rank != dst:
        t = torch.from_numpy(blk)
        dist.send(t.to(dev) if dev is not None else t, dst=dist.get_global_rank(group, dst) if group else dst,
                  group=group)
        return None, (r0, r1, c0, c1)
    C = np.empty((M, N), np.float64)
    C[r0:r1, c0:c1] = blk
    for src in range(world):
        if src == rank:
            continue
        q0, q1, p0, p1 = block_range(src, world, M, N, grid)
        t = torch.empty((q1 - q0, p1 - p0), dtype=torch.float64, device=dev)
        dist.recv(t, src=dist.get_global_rank(group, src) if group else src, group=group)
        C[q0:q1, p0:p1] = t.cpu().numpy()
    return C, (r0, r1, c0, c1)
