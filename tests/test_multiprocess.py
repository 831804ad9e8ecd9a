"""Replica bookkeeping of bench.py on CPU ranks (gloo, world size 2): barrier, max over ranks,
and the whole-job value N x rays / max time. The hair path shards no data across GPUs (rays
are independent; each rank builds its own BVH and renders its own frames)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    assert d.rank == rank and d.world == world
    d.barrier()
    ms = 10.0 + 5.0 * rank          # the slower rank decides the job time
    m = d.max(ms)
    rays_per_rank = 1_000_000
    value = d.world * rays_per_rank / (m * 1e-3) / 1e6
    q.put((rank, m, value))
    d.close()


@pytest.mark.parametrize("world", [2])
def test_replica_max_over_ranks(world):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, m, value in res:
        assert m == 15.0
        assert abs(value - world * 1e6 / 15e-3 / 1e6) < 1e-9


def test_single_process_dist_is_trivial():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    assert d.world == 1 and d.rank == 0 and d.max(3.5) == 3.5
    d.barrier()
    d.close()
