"""The multi-rank path of bench.py on CPU (gloo, world size 2): timing is the
maximum over ranks, every rank simulates its own particles (distinct
seeds: weak scaling with no data-path collective), the job value counts all
ranks' work."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(10.0 + rank)
    seeds = [s.seed for s in bench.workload_sims(1000, rank)]
    dist.destroy_process_group()
    out.put((rank, t, seeds))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]            # max over ranks on every rank
    assert not set(res[0][2]) & set(res[1][2])             # disjoint random streams


def test_weak_scaling_value():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.weak_scaling_value(4_000_000, 5, 1000.0, 2) == pytest.approx(4e7)
    assert bench.max_over_ranks(3.5) == 3.5                # not distributed
