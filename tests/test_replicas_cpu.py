"""The bench's N > 1 path (replicas, one process per GPU): timings reduced to
their maximum over ranks and barriers around the timed region, exercised
with two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.ranks_barrier()
        out = bench.max_over_ranks([10.0 + rank, 5.0 - rank, float(rank)])
        q.put((rank, bench.dist_info(), out))
        bench.ranks_barrier()
    finally:
        dist.destroy_process_group()


def test_timings_reduce_to_the_slowest_replica():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in range(2):
        rank, info, out = q.get(timeout=120)
        got[rank] = (info, out)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert got[r][0] == (r, 2, r)
        assert got[r][1] == [11.0, 5.0, 1.0]


def test_single_process_leaves_timings_alone(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert bench.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    bench.ranks_barrier()  # no process group: nothing to wait for
