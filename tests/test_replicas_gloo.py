"""bench.py's multi-process path on CPU: world_size-2 gloo ranks (the path
runs replicas, one per GPU, so the only exchange is the max-over-ranks of the
timed duration), and the reference arm's non-zero ranks exit without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 * (rank + 1), dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got, bench.dist_env()))


def test_max_over_ranks_with_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]
    assert [r[2][:2] for r in res] == [(0, 2), (1, 2)]


def test_reference_arm_nonzero_rank_exits_quietly(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        n = 2000
        steps = 1
        warmup = 0
        gpus = 2
        cpu_seconds = 1.0
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
