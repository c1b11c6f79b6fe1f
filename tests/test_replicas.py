"""The N > 1 path of bench.py (independent replicas, no device collective) on CPU with gloo,
world size 2: the job time is the max over ranks and the value counts every rank's particles."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, port, q):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    out = {"ms_per_step": [2.0, 3.0][rank], "value": 0.0, "config": {"particles": 1000, "parallelism": "single"}}
    r = bench.reduce_replicas(out, 2, 8)
    dist.destroy_process_group()
    q.put((rank, r["ms_per_step"], r["value"], r["config"]["parallelism"]))


def test_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, par in got:
        assert ms == 3.0
        assert value == pytest.approx(1000 * 8 * 2 / 3.0e-3)
        assert par == "replicas x2"
