"""The N > 1 benchmark path on CPU: two gloo ranks (127.0.0.1) run the replica bookkeeping the benchmark uses
(barrier, max of step times, sum of units)."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from metapart_gb300.replicas import Replicas
    r = Replicas()
    r.barrier()
    q.put((rank, r.max(10.0 * (rank + 1)), r.sum(rank + 1)))
    r.barrier()
    r.close()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 20.0, 3.0), (1, 20.0, 3.0)]
