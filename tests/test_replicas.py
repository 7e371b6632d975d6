"""The multi-GPU path of bench.py is replicas only: independent copies of the
workload per rank, a barrier around the timed region and the max of the
per-rank times.  Its host logic runs here with two gloo ranks on the CPU."""
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
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    m = bench.allmax(w, 10.0 * (rank + 1))
    # the reference arm does its work on rank 0 only
    class A:
        steps, warmup = 1, 0
    out = bench.run_reference(A, w, r, bench.Workload("gresho", 16)) if r != 0 else "skipped"
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((rank, m, out))


def test_two_rank_barrier_and_max():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [20.0, 20.0]
    assert res[1][2] is None
