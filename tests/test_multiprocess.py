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


def _box_step(b, seed=5):
    """one oracle step (push, fixed-point deposit, charge, red-black SOR, E)
    of a small box whose state is drawn from its id: the CPU stand-in for a
    box of the GPU ensemble"""
    import numpy as np
    from oracle import pyoracle as po
    rng = np.random.default_rng(seed * 1000 + b)
    n3 = rng.integers(7, 12, size=3)
    g = po.grid(n3, [-0.1, -0.1, 0.0], [0.1, 0.1, 0.2])
    n = int(rng.integers(200, 2000))
    P = np.zeros((7, n))
    P[0:3] = np.array(g.x0)[:, None] + rng.random((3, n)) * (np.array(g.xm) - np.array(g.x0))[:, None]
    P[3:6] = rng.standard_normal((3, n)) * 3e5
    P[6] = 1e4
    ef = po.efield(g, np.zeros(g.nn))
    P = po.push_box(g, ef, -1.602176565e-19, 9.10938215e-31, 2e-10, P)
    fx = 2.0 ** po.fixed_scale_exponent(1e4, n)
    den = po.density_from_fixed(po.deposit_fixed(g, P, fx), fx, po.node_volumes(g))
    rho = po.charge_density([-1.602176565e-19], den[None, :])
    phi, _, _, _ = po.sor_box(g, np.zeros(g.nn), rho, 10000, 1e-4, "rb")
    return n3, n, P, phi


def _shard_rank(rank, world_size, port, out):
    import sys
    import numpy as np
    import torch.distributed as dist
    from conftest import ROOT
    sys.path.insert(0, ROOT)
    import bench
    E = bench.espic_module()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    # the benchmark's own shard of the 512-box ensemble
    mine512 = bench.ensemble_shard(E, bench.CONFIGS["ensemble512"], rank, world_size)
    # a small ensemble stepped by the oracle, split by the same partitioner
    specs = [_box_step(b)[:2] for b in range(12)]
    nodes = np.array([s[0] for s in specs])
    parts = np.array([s[1] for s in specs])
    owner, load = E.partition_boxes(E.ensemble_work(nodes, parts), world_size)
    mine = np.nonzero(owner == rank)[0]
    res = {int(b): _box_step(int(b))[2:] for b in mine}
    gathered = [None] * world_size
    dist.all_gather_object(gathered, res)
    owned = [None] * world_size
    dist.all_gather_object(owned, [int(b) for b in mine512])
    union = {}
    for g in gathered:
        union.update(g)
    out[rank] = (union, owned, list(load))
    dist.destroy_process_group()


def test_ensemble_sharded_over_two_ranks():
    """bench.py's N>1 ensemble path: every rank runs the partitioner of the
    C-ABI (espic_partition_boxes, no GPU needed) and steps only its boxes,
    with no exchange.  Two gloo ranks: the 512 boxes are owned exactly once
    with balanced work, and the union of the ranks' per-box results (oracle
    box steps standing in for the GPU ensemble) equals the single-rank
    results box by box."""
    import numpy as np
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    union, owned, load = out[0]
    assert sorted(owned[0] + owned[1]) == list(range(512))
    assert not set(owned[0]) & set(owned[1])
    assert max(load) <= 1.1 * min(load)
    assert sorted(union) == list(range(12))
    for b in range(12):
        P, phi = _box_step(b)[2:]
        assert np.array_equal(union[b][0], P) and np.array_equal(union[b][1], phi)
