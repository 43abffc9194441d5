"""Multi-rank path of bench.py on CPU (gloo, world size 2).

The matmul path shards as replicas (every rank multiplies its own
problems; no data-path collective), so the only cross-rank logic is the
barrier around the timed region and the max-over-ranks of the step time,
which bench.py's helpers implement for both NCCL (GPU) and gloo (CPU).
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    worst = bench.max_over_ranks(1.0 + rank, w)      # per-rank step times
    total = bench.sum_over_ranks(10.0, w)           # units processed
    out[rank] = (worst, total)
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert out[0] == out[1] == (2.0, 20.0)
