"""The N>1 path of bench.py: independent replicas, one per rank, with the
step time taken as the maximum over ranks and the throughput as the units of
all ranks over that time.  Run here as world_size-2 gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world_size, port, out):
    import sys
    import torch.distributed as dist
    from conftest import ROOT
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    ms = [3.0, 5.0][rank]
    n = [4.0e6, 3.0e6][rank]
    res = bench.aggregate(ms, n, dist, "cpu")
    out[rank] = res
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        ms, value, ws = out[r]
        assert ws == 2 and ms == 5.0
        assert value == pytest.approx(7.0e6 / 5e-3)


def test_single_rank_aggregation():
    from conftest import ROOT
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate(2.0, 1e6, None, "cpu") == (2.0, 1e6 / 2e-3, 1)
