"""The N > 1 path of bench.py on CPU: world_size 2 over gloo, as torchrun
launches it (one process per GPU, replicas only).  Each rank must see the
max over ranks of its step time, the barrier must hold, and the whole-job
value is world x solves/s of the slowest replica.  No GPU is touched
(select_device=False); the device choice itself is LOCAL_RANK."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, barrier, vmax = bench.dist_init(world, select_device=False)
    ms = 100.0 + 50.0 * r  # rank 1 is the slower replica
    barrier()
    m = vmax(ms)
    value = bench.aggregate(w, m)
    barrier()
    with open(os.path.join(out, "rank%d.json" % r), "w") as f:
        json.dump({"rank": r, "world": w, "max_ms": m, "value": value}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_over_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    for r in res:
        assert r["world"] == world
        assert r["max_ms"] == 150.0          # the slowest replica's time on every rank
        assert abs(r["value"] - world * 1000.0 / 150.0) < 1e-9


def test_single_process_path():
    sys.path.insert(0, ROOT)
    import bench
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        r, w, barrier, vmax = bench.dist_init(1)
        assert (r, w) == (0, 1) and vmax(3.5) == 3.5
        barrier()
        assert bench.aggregate(1, 250.0) == 4.0
    finally:
        os.environ.update(env)
