"""Splitting a sweep across ranks (one GPU per rank): two gloo ranks on the CPU compute their
shares of the 4096-instance batch independently; together they cover every instance once, with
balanced predicted cost."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "py-fdtd_pic_gb300"))
    import torch.distributed as dist
    from fdtdpic import sweep
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    spec = sweep.SweepSpec(n_inst=4096, n_steps=64)
    params = sweep.sweep_parameters(spec)
    # cheap stand-ins with the batch's costs (the full grids are not needed to split it)
    from types import SimpleNamespace
    costs = [64 * (p["nz"] + 12.0 * (p["rear"] - p["front"])) for p in params]
    grids = [SimpleNamespace(cost=(lambda c=c: c)) for c in costs]
    mine = sweep.shard_indices(grids, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, sum(costs[i] for i in mine)))
    if rank == 0:
        out.put(gathered)
    dist.destroy_process_group()


def test_two_ranks_cover_the_sweep_once():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (a, ca), (b, cb) = gathered
    assert sorted(a + b) == list(range(4096))
    assert not set(a) & set(b)
    assert abs(ca - cb) / (ca + cb) < 0.01
