"""Multi-process path of bench.py on CPU (gloo, world size 2): with N GPUs the
benchmark runs N independent replicas; the only cross-rank traffic is the
barrier around the timed region and the max-over-ranks of the step time."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        q.put((rank, d.max(10.0 * (rank + 1)), d.world))
    finally:
        d.close()


def test_two_rank_max_and_barrier():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 20.0, 2), (1, 20.0, 2)]
