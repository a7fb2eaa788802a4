"""The multi-rank plumbing of bench.py (replicas: one rank per GPU, no
exchange on the data path), exercised with two gloo ranks on the CPU: the
process-group setup from the torchrun environment, the timing barrier and
the max-over-ranks reduction that turns per-rank times into the job's time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup(world, backend="gloo")
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + r, w)        # rank r "took" 1 + r seconds
    bench.barrier(w)
    q.put((r, w, local, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 2.0 for o in out)     # both ranks report the max


def test_single_rank_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench.dist_setup(1) == (0, 1, 0)
    assert bench.max_over_ranks(3.5, 1) == 3.5
