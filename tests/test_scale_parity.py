"""Bit-exact parity at the benchmarked sizes.

The reference's TSV output over these inputs runs to tens of millions of lines
(the small read set at its full 138 Mbp, the repetitive assembly and the k=63
read set at 1/10 of their 3.1 / 3 Gbp), too many to store as fixtures. The
reference binaries' output was recorded as an order-independent digest of the
(k-mer, count) pairs (oracle/tuna_digest.h), with the line count and the
superkmers: value (tests/golden/make_golden.py --scale). The GPU path must give
the same digest through tg_job_result_digest, which hashes the pairs on the
device with the library's own code.

CPU tests pin the digest itself: the oracle's digest of its own pairs equals
the digest the C digester computes from the reference's committed TSV lines,
and the oracle's digest pipeline equals the reference's digest at full size.
"""
import os

import pytest

from tests import golden_util as G

U64_MAX = (1 << 64) - 1
SCALE = ["scale_reads_k31_m21", "scale_rep_fasta_k31_m23", "scale_large_k63_m21"]


@pytest.fixture(scope="module")
def ctx():
    import tuna_gb300 as T
    c = T.Context(0, autotune=True)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCALE)
def test_scale_digest_fastx(ctx, name):
    """FASTA/FASTQ bytes lexed and counted on the device; digest, pair count and
    record count equal the reference's."""
    fx = G.fixture(name)
    data = G.case_input(name)  # regenerated from its seed, sha256 checked
    cx = fx["cx"] if fx["cx"] is not None else U64_MAX
    r, _ = ctx.run(fx["k"], fx["m"], fastx=data, n_parts=fx["n"], ci=fx["ci"], cx=cx, want_results=False,
                   digest=True)
    assert r.stats["superkmers"] == fx["reference_stderr"]["superkmers"]
    assert r.stats["out"] == fx["lines"]
    assert r.digest == fx["digest"], f"{name}: GPU {r.digest} vs reference {fx['digest']}"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["scale_reads_k31_m21", "scale_large_k63_m21"])
def test_scale_digest_passes(name):
    """The same digest when phase 2 runs in passes under a small memory budget
    (the pairs then sit in host memory and are digested on host threads)."""
    import tuna_gb300 as T
    fx = G.fixture(name)
    data = G.case_input(name)
    cx = fx["cx"] if fx["cx"] is not None else U64_MAX
    with T.Context(0, hbm_budget=1 << 30) as c:
        r, _ = c.run(fx["k"], fx["m"], fastx=data, n_parts=fx["n"], ci=fx["ci"], cx=cx, want_results=False,
                     digest=True)
    assert r.stats["phase2_passes"] > 1
    assert r.digest == fx["digest"]


@pytest.mark.gpu
def test_scale_digest_matches_copied_pairs(ctx):
    """The device digest equals the oracle's digest of the same pairs copied to
    the host (the two implementations of the digest agree)."""
    from oracle import oracle as O
    fx = G.fixture("scale_large_k63_m21")
    data = G.case_input("scale_large_k63_m21")
    r, _ = ctx.run(63, 21, fastx=data, n_parts=64, ci=2, cx=10000, digest=True)
    assert O.digest_pairs(r.keys, r.counts, 63) == r.digest == fx["digest"]


def test_digest_of_reference_tsv_lines():
    """The C digester over the reference's own TSV lines (committed fixtures)
    equals the oracle's digest of its pairs for the same input: the digest is
    pinned on the reference's bytes, k from 5 to 63."""
    import tempfile
    from oracle import oracle as O
    for name in ["edge_fasta_k5", "edge_fasta_k31", "edge_fasta_k63", "fuzz_fasta_k33", "fuzz_fastq_k15",
                 "ci_smoke_k31"]:
        fx = G.fixture(name)
        tsv = G.full_tsv(name)
        with tempfile.NamedTemporaryFile(suffix=".tsv", delete=False) as f:
            f.write(tsv)
            path = f.name
        try:
            ref = O.tsv_digest_file(path)
        finally:
            os.remove(path)
        data = G.case_input(name)
        cx = fx["cx"] if fx["cx"] is not None else U64_MAX
        res = O.count_fastx(data, fx["k"], fx["m"], fx["n"], fx["ci"], cx, threads=2)
        assert O.digest_pairs(res.keys, res.counts, fx["k"]) == ref, name
        assert ref["pairs"] == fx["lines"]


@pytest.mark.parametrize("name", ["scale_reads_k31_m21", "scale_large_k63_m21"])
def test_oracle_digest_at_scale(name):
    """The oracle's digest pipeline (no pairs kept) equals the reference's
    digest at the recorded sizes (138 Mbp of reads; 300 Mbp of k=63 reads)."""
    from oracle import oracle as O
    fx = G.fixture(name)
    data = G.case_input(name)
    cx = fx["cx"] if fx["cx"] is not None else U64_MAX
    d, st = O.digest_stream(data, fx["k"], fx["m"], fx["n"], fx["ci"], cx, threads=os.cpu_count() or 1,
                            fastx=True)
    assert st["n_superkmers"] == fx["reference_stderr"]["superkmers"]
    assert d == fx["digest"]
