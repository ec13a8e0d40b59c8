"""The N > 1 path of bench.py on CPU: two gloo ranks on 127.0.0.1 run the
replica coordination (process group from the torchrun environment, barrier,
max of the step times over ranks)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, local = bench.replicas()
    bench.barrier(w)
    step_s = 1.5 + r  # each replica's own time
    out.put((r, w, local, bench.max_over_ranks(step_s, w), os.environ["CUDA_VISIBLE_DEVICES"]))
    dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_step():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    assert all(g[1] == 2 for g in got)
    assert all(g[3] == 2.5 for g in got)  # the max over ranks
    assert [g[4] for g in got] == ["0", "1"]  # one GPU per replica


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.replicas() == (1, 0, 0)
    assert bench.max_over_ranks(3.25, 1) == 3.25
