"""The N > 1 bench path: independent replicas, a barrier around the timed region and the maximum
step time over ranks. Run as two gloo ranks on the CPU (no GPU, no data-path collective)."""
import os
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    v = bench.allmax(10.0 + rank, world)  # each replica reports its own step time
    out[rank] = v
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world, port = 2, 29517
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    assert dict(out) == {0: 11.0, 1: 11.0}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.allmax(3.5, 1) == 3.5
    bench.barrier(1)
