"""Multi-rank host logic on CPU (gloo, world size 2): the bench's max-over-ranks
timing, and the reference arm under torchrun, where rank 0 alone runs and prints.

With N GPUs each rank runs its own DGEMM (weak scaling, no data-path
collective); the only collective is the MAX of the per-rank step time.
"""
import json
import os
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _worker(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    v = bench.max_over_ranks(1.5 + 3.0 * rank)
    out.put((rank, v))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 4.5, 1: 4.5}


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.0) == 2.0


def test_reference_arm_two_ranks_prints_one_line():
    """bench.py --impl reference under torchrun with 2 ranks: one JSON line (rank 0),
    both ranks exit 0."""
    port = 30500 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["higher_is_better"] is True and d["unit"] == "TFLOP/s"
