"""Multi-GPU runs are replicas (one independent solve per rank, no data-path
collective): the benchmark's rank coordination -- barrier, max and sum over
ranks of the timings -- on world_size 2 with the gloo backend on CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    wsz, rk, local = bench.dist_env()
    d = bench.Dist(wsz)
    d.barrier()
    mx = d.max(1.0 + rank)          # per-rank seconds -> the slowest rank
    sm = d.sum(3.0)                 # per-rank units -> the whole job's units
    d.barrier()
    out[rank] = (wsz, rk, local, mx, sm)
    torch.distributed.destroy_process_group()


def test_dist_max_and_sum_over_two_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        out = man.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == (2, 0, 0, 2.0, 6.0)
    assert res[1] == (2, 1, 1, 2.0, 6.0)
