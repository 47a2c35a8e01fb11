"""Multi-GPU runs are independent replicas: bench.py's whole-job figures are the
slowest rank's time and the sum of all ranks' units.  Checked with two gloo ranks
on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_ms = [120.0, 95.5][rank]          # per-rank timed region
        units = [500, 450][rank]            # RHS-iterations each rank did
        t, u = bench.aggregate_replicas(torch, t_ms, units, "cpu")
        out[rank] = (t, u, bench.dist_info())
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    pytest.importorskip("torch.distributed")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        t, u, info = res[r]
        assert t == 120.0 and u == 950.0
        assert info == (r, world, 0)
