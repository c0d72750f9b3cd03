"""The multi-GPU form of the bench is N independent replicas (one process
per GPU, no data-path collective): what the processes share is a barrier
and the max of their step times.  Checked here with world_size-2 gloo
process groups on the CPU."""
import os
import socket
import sys
from pathlib import Path

import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        impl = "reference"  # gloo process group (the GPU arm uses NCCL)

    w, r, local = bench.dist_setup(Args)
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    # each replica reports its own step time; every rank sees the slowest
    slowest = bench.max_over_ranks(1.5 + rank, w, torch.device("cpu"))
    out[rank] = slowest
    bench.barrier(w)
    torch.distributed.destroy_process_group()


def test_two_replicas_barrier_and_max_over_ranks():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert dict(out) == {0: 1.5 + world - 1, 1: 1.5 + world - 1}


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        impl = "ours"

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        assert bench.dist_setup(Args) == (1, 0, 0)
        assert bench.max_over_ranks(3.25, 1, torch.device("cpu")) == 3.25
    finally:
        os.environ.update(env)
