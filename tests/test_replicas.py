"""The multi-GPU path is replicas only: every rank runs its own tank and the
benchmark reports all ranks' particle-steps over the slowest rank's time.
Two gloo ranks on the CPU check that plumbing (bench.Dist, bench.aggregate):
the barrier, the max over ranks, and the whole-job throughput."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BSC_DIST_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    # rank r took 1 + r seconds for 1000 particle-steps
    value, tmax = bench.aggregate(1.0 + rank, 1000.0, d)
    out.put((rank, d.world, value, tmax))
    d.close()


def test_two_gloo_replicas_aggregate():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, world, value, tmax in res:
        assert world == 2
        assert tmax == 2.0                   # the slowest rank's time
        assert value == 2 * 1000.0 / 2.0     # both ranks' units over it
