"""The shard rule of tg_job_set_shard restated with the oracle, on CPU.

For a job of one sample a k-mer's bin is its record's minimizer hash modulo
2^20, which is the oracle's partition id with 2^20 partitions; shard s of n
holds bins [s 2^20 / n, (s + 1) 2^20 / n). The pairs of each shard, read back
from the oracle's records, are disjoint, and together they are the oracle's
count of the whole input: in one process, and across two gloo ranks that each
count one shard and exchange their pairs (the host side of a job split over
two devices, where nothing else crosses between them).
"""
import os
import socket
import sys
from collections import Counter

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BINS = 1 << 20
_COMP = bytes.maketrans(b"ACGT", b"TGCA")


def _input():
    from tuna_gb300 import synth
    g = synth.genome(150_000, 17, 0.45, fam_a=(30, 300, 0.05), div=(0.0, 0.03))
    return bytes(g[:80_000]) + b"\n" + bytes(g[60_000:]) + b"\n"  # an overlap repeats k-mers


def shard_pairs(parts, k: int, m: int, shard: int, n: int) -> Counter:
    """Canonical k-mer counts of the records in bins of shard `shard` of `n`."""
    from oracle import oracle as O
    out = Counter()
    lo, hi = shard * BINS // n, (shard + 1) * BINS // n
    for p in range(lo, hi):
        if not parts[p]:
            continue
        for ln, _mp, packed in O.split_records(parts[p], k, m):
            seq = bytes(b"ACGT"[(packed[i >> 2] >> (6 - 2 * (i & 3))) & 3] for i in range(ln))
            for i in range(ln - k + 1):
                f = seq[i:i + k]
                out[min(f, f.translate(_COMP)[::-1])] += 1
    return out


def _oracle_pairs(seq, k, m) -> Counter:
    from oracle import oracle as O
    r = O.count_stream(seq, k, m, n_parts=16)
    out = Counter()
    for ln in r.tsv_lines():
        km, c = ln.split("\t")
        out[km.encode()] = int(c)
    return out


@pytest.mark.parametrize("k,m,n", [(31, 21, 2), (31, 21, 16), (25, 21, 4), (63, 21, 8)])
def test_shards_are_disjoint_and_complete(k, m, n):
    from oracle import oracle as O
    seq = _input()
    parts = O.partition_stream(seq, k, m, BINS)
    shards = [shard_pairs(parts, k, m, s, n) for s in range(n)]
    for a in range(n):
        for b in range(a + 1, n):
            assert not (shards[a].keys() & shards[b].keys()), (a, b)
    union = Counter()
    for s in shards:
        union.update(s)
    assert union == _oracle_pairs(seq, k, m)
    assert all(shards)  # every shard holds pairs at this size


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seq = _input()
        mine = shard_pairs(O.partition_stream(seq, 31, 21, BINS), 31, 21, rank, world)
        everyone = [None] * world
        dist.all_gather_object(everyone, dict(mine))
        if rank == 0:
            keys = [set(d) for d in everyone]
            disjoint = not (keys[0] & keys[1])
            union = Counter()
            for d in everyone:
                union.update(d)
            q.put((disjoint, union == _oracle_pairs(seq, 31, 21), [len(d) for d in everyone]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_one_shard_each_gloo():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    disjoint, complete, sizes = q.get(timeout=10)
    assert disjoint and complete and all(sizes)
