"""Multi-GPU replicas on CPU: two gloo ranks (world_size 2, 127.0.0.1) take
the max of their step times and compute the whole-job throughput; replica
scenes differ only in their jitter seed."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import nullpath_gb300 as npx
from nullpath_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 100.0 + 25.0 * rank
    mx = replicas.max_over_ranks(ms)
    v = replicas.aggregate_rays_per_s(1000.0, mx, ws)
    q.put((rank, mx, v, replicas.rank_scene(npx.benchmark_scene(width=8, height=8), rank).seed))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [125.0, 125.0]
    assert all(abs(o[2] - 2 * 1000.0 / 0.125) < 1e-9 for o in out)
    assert [o[3] for o in out] == [0, 1]


def test_single_process_is_identity():
    assert replicas.max_over_ranks(3.5) == 3.5
    a = npx.benchmark_scene(width=8, height=8, seed=4)
    b = replicas.rank_scene(a, 3)
    assert b.seed == 7 and (b.width, b.spin, b.theta_deg) == (a.width, a.spin, a.theta_deg)
