"""Replica aggregation across ranks (gloo, world size 2, CPU only): the
whole-job throughput is the sum of the ranks' work over the slowest rank's
time, and a rank's environment is read from the torchrun variables."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from sw2_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        env = replicas.dist_env()
        # rank r did (r+1) * 1e6 cell-updates in (r+1) * 0.5 s
        thr, total, tmax = replicas.aggregate((rank + 1) * 1e6, (rank + 1) * 0.5)
        q.put((rank, env, thr, total, tmax))
    finally:
        dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, env, thr, total, tmax in out:
        assert env == (ws, rank, rank)
        assert total == 3e6 and tmax == 1.0 and thr == 3e6


def test_aggregate_single_process():
    thr, total, tmax = replicas.aggregate(5e6, 2.0)
    assert (thr, total, tmax) == (2.5e6, 5e6, 2.0)
