"""GPU path against the reference (golden fixtures) and the oracle.

Bit-exact is the bar: the sorted TSV bytes of the GPU output must hash to the
reference's, record counts must match the reference's superkmers: line, and
exported Phase 1 partitions must hold the same record multisets.
"""
import numpy as np
import pytest

from tests import golden_util as G

pytestmark = pytest.mark.gpu

U64_MAX = (1 << 64) - 1


@pytest.fixture(scope="module")
def ctx():
    import tuna_gb300 as T
    c = T.Context(0)
    yield c
    c.close()


def _gpu_cases():
    out = []
    for n in G.CASE_NAMES:
        fx = G.fixture(n)
        if fx["k"] <= 63:
            out.append(n)
    return out


@pytest.mark.parametrize("name", _gpu_cases())
def test_golden_counts(ctx, name):
    import tuna_gb300 as T
    fx = G.fixture(name)
    data = G.case_input(name)
    cx = fx["cx"] if fx["cx"] is not None else U64_MAX
    r, _ = ctx.run(fx["k"], fx["m"], fastx=data, n_parts=fx["n"], ci=fx["ci"], cx=cx)
    blob = T.tsv_blob(r.keys, r.counts, fx["k"])
    full = G.full_tsv(name)
    if full is not None and blob != full:
        got, want = set(blob.split(b"\n")), set(full.split(b"\n"))
        pytest.fail(f"{name}: {len(got - want)} extra, {len(want - got)} missing: "
                    f"{sorted(got - want)[:3]} / {sorted(want - got)[:3]}")
    assert len(r) == fx["lines"]
    assert G.sha(blob) == fx["tsv_sha256"]
    assert r.stats["superkmers"] == fx["reference_stderr"]["superkmers"]


@pytest.mark.parametrize("name", [n for n in _gpu_cases() if G.parts_fixture(n)])
def test_golden_partitions(ctx, name):
    from oracle.oracle import split_records
    pj = G.parts_fixture(name)
    data = G.case_input(name)
    _, parts = ctx.run(pj["k"], pj["m"], fastx=data, n_parts=pj["n"], export=True, want_results=False)
    for p, want in enumerate(pj["partitions"]):
        recs = split_records(parts[p], pj["k"], pj["m"])
        assert len(recs) == want["records"], f"partition {p}"
        assert len(parts[p]) == want["bytes"], f"partition {p}"
        assert G.record_multiset_sha(recs) == want["sha256"], f"partition {p}"


@pytest.mark.parametrize("gpu_parts", [1, 16, 512, 4096])
def test_bucket_count_does_not_change_output(ctx, gpu_parts):
    import tuna_gb300 as T
    name = "reads_k31_m21"
    fx = G.fixture(name)
    data = G.case_input(name)
    r, _ = ctx.run(31, 21, fastx=data, gpu_parts=gpu_parts)
    assert G.sha(T.tsv_blob(r.keys, r.counts, 31)) == fx["tsv_sha256"]


def test_stream_equals_fastx(ctx):
    """The host parser's stream and a stream built by the oracle's parser give
    the same counts."""
    from oracle import oracle as O
    import tuna_gb300 as T
    data = G.case_input("fuzz_fastq_k31")
    stream = O.fastx_to_stream(data)
    a, _ = ctx.run(31, 21, fastx=data)
    b, _ = ctx.run(31, 21, seq=stream)
    assert T.tsv_blob(a.keys, a.counts, 31) == T.tsv_blob(b.keys, b.counts, 31)


def test_device_feed_matches_host_feed(ctx):
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.005, seed=3)
    stream = synth.fastq_sequence_stream(fq)
    d = torch.from_numpy(stream).to("cuda:0")
    torch.cuda.synchronize()
    a, _ = ctx.run(31, 21, dev_seq=d.data_ptr(), dev_len=d.numel())
    b, _ = ctx.run(31, 21, seq=stream)
    assert T.tsv_blob(a.keys, a.counts, 31) == T.tsv_blob(b.keys, b.counts, 31)


@pytest.mark.parametrize("k,m", [(31, 21), (31, 23), (63, 21), (21, 17), (25, 21), (32, 21), (33, 21),
                                 (2, 1), (5, 3), (47, 31), (63, 32)])
def test_against_oracle(ctx, k, m):
    from oracle import oracle as O
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g = synth.genome(60_000, 5, 0.45, fam_a=(5, 300, 0.3), div=(0.02, 0.05), micro=0.05)
    fa = synth.fasta(g, [20_000, 25_000, 15_000])
    want = O.count_fastx(fa, k, m, n_parts=16, threads=4)
    got, _ = ctx.run(k, m, fastx=fa)
    assert got.stats["superkmers"] == want.stats["n_superkmers"]
    assert got.stats["kmers"] == want.stats["n_kmers"]
    assert got.stats["distinct"] == want.stats["n_distinct"]
    assert T.tsv_blob(got.keys, got.counts, k) == O.tsv_blob(want)


def test_ci_cx_filter(ctx):
    from oracle import oracle as O
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.003, seed=9)
    for ci, cx in [(2, U64_MAX), (1, 5), (3, 3), (100, 200)]:
        want = O.count_fastx(fq, 31, 21, ci=ci, cx=cx, threads=4)
        got, _ = ctx.run(31, 21, fastx=fq, ci=ci, cx=cx)
        assert T.tsv_blob(got.keys, got.counts, 31) == O.tsv_blob(want), (ci, cx)


def test_filter_equals_post_filter(ctx):
    """-ci/-cx inside the count kernel keep exactly the pairs that filtering the
    unfiltered output afterwards keeps (the reference applies the bounds as each
    bin's table is drained, src/count.hpp:270-287)."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.003, seed=21)
    full, _ = ctx.run(31, 21, fastx=fq)
    assert len(full) > 0
    for ci, cx in [(2, 40), (1, 1), (4, U64_MAX), (7, 9)]:
        got, _ = ctx.run(31, 21, fastx=fq, ci=ci, cx=cx)
        keep = (full.counts >= ci) & (full.counts.astype(np.uint64) <= np.uint64(cx))
        assert T.tsv_blob(got.keys, got.counts, 31) == \
            T.tsv_blob(full.keys[keep], full.counts[keep], 31), (ci, cx)


def test_empty_and_separator_only(ctx):
    r, _ = ctx.run(31, 21, seq=b"NNNN\n\n\r")
    assert len(r) == 0
    r, _ = ctx.run(31, 21, seq=b"ACGT" * 7)  # 28 bases < k
    assert len(r) == 0 and r.stats["kmers"] == 0


def test_poly_a_and_long_chains(ctx):
    """Long runs with a constant minimizer: records are cut every 256 - k
    k-mers (forced splits) and chains cross Phase-1 CTA chunks."""
    from oracle import oracle as O
    import tuna_gb300 as T
    seq = b"A" * 300_000 + b"N" + b"AC" * 200_000 + b"\n" + b"ACGTTGCA" * 50_000
    want = O.count_stream(seq, 31, 21, n_parts=16)
    got, parts = ctx.run(31, 21, seq=seq, export=True, n_parts=16)
    assert got.stats["superkmers"] == want.stats["n_superkmers"]
    assert T.tsv_blob(got.keys, got.counts, 31) == O.tsv_blob(want)
    ref_parts = O.partition_stream(seq, 31, 21, 16)
    for p in range(16):
        assert sorted(O.split_records(parts[p], 31, 21)) == sorted(O.split_records(ref_parts[p], 31, 21))
