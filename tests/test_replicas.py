"""Multi-GPU runs are independent replicas (one scene per rank, no exchange between them): the only
host logic across ranks is the job-level rate, the units of all ranks over the slowest rank's time.
Checked here with two gloo processes on the CPU."""
import os
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        value, ms = bench.job_rate(10.0 * (rank + 1), 1000, world, "cpu")  # rank 1 is the slower one
        out[rank] = (value, ms)
    finally:
        dist.destroy_process_group()


def test_job_rate_takes_the_slowest_rank():
    world = 2
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        value, ms = res[r]
        assert ms == 20.0
        assert abs(value - 2 * 1000 / 0.020) < 1e-6
