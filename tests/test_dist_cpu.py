"""The multi-GPU path of bench.py on CPU: two gloo ranks.

The solver is replicas-only (every GPU solves its own system; no data-path
collective).  The bench's timing needs a barrier around the timed region and
the maximum of the per-rank times; these run here on world_size 2."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(world)
    d.barrier()
    m = d.max(1.5 + rank)  # per-rank "seconds"
    d.barrier()
    q.put((rank, d.rank, d.world, m))
    d.close()


def test_two_rank_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [0, 1] and all(r[2] == 2 for r in res)
    assert all(r[3] == 2.5 for r in res)  # every rank sees the slowest rank's time
    assert all(p.exitcode == 0 for p in procs)
