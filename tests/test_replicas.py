"""Multi-rank (replica) bookkeeping on CPU with gloo, world size 2."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    from convstencil_gb300 import replicas
    replicas.init("gloo")
    # rank r processed (r+1)*1e9 point-steps in (r+1) seconds
    thr, t = replicas.job_throughput((rank + 1) * 1e9, float(rank + 1))
    replicas.barrier()
    q.put((rank, thr, t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_throughput_uses_total_work_and_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, thr, t in res:
        assert t == 2.0                       # slowest rank
        assert thr == pytest.approx(3e9 / 2)  # all ranks' work / slowest time


def test_single_process_is_identity():
    from convstencil_gb300 import replicas
    assert replicas.job_throughput(5.0, 2.0) == (2.5, 2.0)
