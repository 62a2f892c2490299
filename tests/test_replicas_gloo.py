"""Multi-process path of bench.py on CPU: two gloo ranks (replicas) agree on the barrier and on
the whole-job rate (all ranks' particle-steps over the slowest rank's time)."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, _ = bench.dist_env()
    d = bench.Dist(w)
    d.barrier()
    ms = 10.0 * (rank + 1)          # rank 1 is the slower one
    n = 1000 * (rank + 1)
    rate, ms_max = bench.whole_job_rate(d, n, 5, ms)
    d.barrier()
    d.close()
    q.put((r, rate, ms_max))


def test_two_gloo_replicas():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # (1000 + 2000) particles x 5 steps over the slower rank's 20 ms
    for r, rate, ms_max in res:
        assert ms_max == 20.0
        assert rate == pytest.approx(3000 * 5 / 0.020)
