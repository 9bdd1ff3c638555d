"""Shards of one job's bins (tg_job_set_shard): the partition -> device map of
a multi-device job, run here shard after shard on one device. Every instance
of a canonical k-mer falls in the same bin, so the shards' pairs are disjoint
and together exactly the job's pairs; each shard runs Phase 1 over the whole
input and Phase 2 over its share of the bins only."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U64_MAX = (1 << 64) - 1


@pytest.fixture(scope="module")
def ctx():
    import tuna_gb300 as T
    c = T.Context(0)
    yield c
    c.close()


def _union_blob(parts, k):
    import tuna_gb300 as T
    keys = np.concatenate([p.keys for p in parts])
    counts = np.concatenate([p.counts for p in parts])
    return T.tsv_blob(keys, counts, k)


@pytest.mark.parametrize("k,m,n", [(31, 21, 2), (31, 21, 4), (63, 21, 4), (25, 21, 16), (21, 17, 1)])
def test_shards_together_are_the_job(ctx, k, m, n):
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.003, seed=5)
    full, _ = ctx.run(k, m, fastx=fq)
    parts = [ctx.run(k, m, fastx=fq, shard=(s, n))[0] for s in range(n)]
    assert sum(len(p) for p in parts) == len(full)
    assert _union_blob(parts, k) == T.tsv_blob(full.keys, full.counts, k)
    for p in parts:
        assert p.stats["kmers"] == full.stats["kmers"]  # Phase 1 saw the whole input
        assert p.stats["superkmers"] == full.stats["superkmers"]
    assert sum(p.stats["distinct"] for p in parts) == full.stats["distinct"]
    if n > 1:
        assert all(0 < len(p) < len(full) for p in parts)


def test_shards_with_filter_oracle(ctx):
    """-ci/-cx per shard, the union against the oracle."""
    from oracle import oracle as O
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.003, seed=11)
    want = O.count_fastx(fq, 31, 21, ci=2, cx=40, threads=4)
    parts = [ctx.run(31, 21, fastx=fq, ci=2, cx=40, shard=(s, 8))[0] for s in range(8)]
    assert _union_blob(parts, 31) == O.tsv_blob(want)


def test_shard_in_passes():
    """A shard larger than the memory budget runs its bins in passes."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g = synth.genome(3_000_000, 3, 0.45, fam_a=(20, 300, 0.1), div=(0.02, 0.08))
    with T.Context(0) as big:
        want, _ = big.run(31, 21, seq=g)
    parts = []
    with T.Context(0, hbm_budget=12 << 20) as small:
        for s in range(2):
            r, _ = small.run(31, 21, seq=g, shard=(s, 2))
            assert r.stats["phase2_passes"] > 1
            parts.append(r)
    assert _union_blob(parts, 31) == T.tsv_blob(want.keys, want.counts, 31)


def test_shard_arguments(ctx):
    import tuna_gb300 as T
    seq = b"ACGTTGCAAC" * 100
    for bad in [(0, 3), (2, 2), (0, 0), (0, 2048)]:
        with pytest.raises(T.GpuError):
            ctx.run(31, 21, seq=seq, shard=bad)
    with pytest.raises(T.GpuError):  # more shards than the requested segments
        ctx.run(31, 21, seq=seq, gpu_parts=16, shard=(0, 32))
    with pytest.raises(T.GpuError):  # a job of several samples
        ctx.run(31, 21, samples=[seq, seq], shard=(0, 2))
    r, _ = ctx.run(31, 21, seq=seq, gpu_parts=64, shard=(63, 64))  # a valid shard still runs afterwards
    assert r.stats["kmers"] == len(seq) - 30
