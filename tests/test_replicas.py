"""The multi-GPU form of bench.py is N independent replicas of the single-GPU stage (the
library's phases exchange no halos across GPUs; the box-sharding layer is
maestroex_gb300/partition.py, tests/test_partition.py): the host logic that combines the
ranks -- the slowest rank's time and the whole-job throughput -- checked with two gloo
processes on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = bench.max_over_ranks(100.0 + 25.0 * rank, ws, device="cpu")
    out[rank] = (ms, bench.job_value(1 << 24, ws, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_cells():
    ws, port = 2, 29641
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    for r in range(ws):
        ms, value = res[r]
        assert ms == 125.0
        assert value == pytest.approx(2 * (1 << 24) / 0.125)
