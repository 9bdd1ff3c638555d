"""The multi-process host logic of bench.py on CPU (gloo, world size 2): the
barrier and the max over ranks that make a step's time the slowest replica's,
and the reference arm, which rank 0 alone runs (other ranks exit without
work). Replicas share no data on the counting path, so this is all the
cross-rank logic there is."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.rank_barrier(world)
        q.put((rank, bench.rank_max(10.0 * (rank + 1), world, "cpu")))
        bench.rank_barrier(world)
    finally:
        dist.destroy_process_group()


def test_rank_max_and_barrier_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 20.0), (1, 20.0)]


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.rank_max(3.5, 1, "cpu") == 3.5
    bench.rank_barrier(1)


def test_reference_arm_other_ranks_do_no_work(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        gpus, steps, warmup, cpu_shard_mbp = 2, 1, 0, 1.0

    bench.run_reference(A(), rank=1)
    assert capsys.readouterr().out == ""
