"""Spill mode (tg_job_set_spill): the job's input in chunks, each chunk's
superkmer records moved to per-bucket streams in host memory or in files, phase
2 in passes over buckets read back. The pairs must be exactly those of the
same job counted in one piece, and of the reference (digest fixtures) at the
benchmarked 138 Mbp size."""
import os

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


def _reads(glen, seed, n_reads):
    from tuna_gb300 import synth
    g = synth.genome(glen, seed, 0.45, fam_a=(20, 600, 0.1), div=(0.03, 0.08), micro=0.02)
    return synth.reads_fastq(g, n_reads, (100, 250), 0.005, 0.0005, seed + 1)


def _same(a, b):
    a, b = a.sorted(), b.sorted()
    return len(a) == len(b) and np.array_equal(a.keys, b.keys) and np.array_equal(a.counts, b.counts)


@pytest.mark.parametrize("k,m,ci,cx", [(31, 21, 1, U64_MAX), (63, 21, 2, 1000), (21, 17, 1, U64_MAX),
                                       (25, 21, 3, U64_MAX)])
def test_spill_in_memory_equals_one_piece(ctx, k, m, ci, cx):
    """A sequence stream fed in one call, cut into ~40 chunks of 256 KiB at run
    separators: the same pairs and the same record and k-mer totals."""
    from tuna_gb300 import synth
    stream = synth.fastq_sequence_stream(_reads(600_000, 7 + k, 60_000))
    want, _ = ctx.run(k, m, seq=stream, ci=ci, cx=cx)
    got, _ = ctx.run(k, m, seq=stream, ci=ci, cx=cx, spill=(256 << 10,))
    assert _same(got, want)
    for key in ("kmers", "superkmers", "runs", "bases", "out", "distinct"):
        assert got.stats[key] == want.stats[key], key
    assert got.stats["record_bytes"] > 0


def test_spill_to_files_many_feeds(ctx, tmp_path):
    """Many feeds (FASTA files lexed on the device, cut before records), bucket
    files under a directory, several phase-2 passes under a small budget; the
    files are gone when the job ends."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g = synth.genome(2_000_000, 91, 0.41, fam_a=(50, 300, 0.2), div=(0.1, 0.2), micro=0.03)
    lens = [50_000] * 40
    fa = synth.fasta(g, np.array(lens, dtype=np.uint64)).tobytes()
    want, _ = ctx.run(31, 23, fastx=fa, n_parts=256)
    d = tmp_path / "spill"
    d.mkdir()
    with T.Context(0, hbm_budget=64 << 20) as c2:
        got, _ = c2.run(31, 23, fastx=fa, n_parts=256, spill=(300_000, str(d)), gpu_parts=128)
    assert _same(got, want)
    assert got.stats["phase2_passes"] > 1
    assert got.stats["superkmers"] == want.stats["superkmers"]
    assert not list(d.iterdir())


def test_spill_full_size_reads_digest(ctx):
    """The small read set at its full 138 Mbp, as a sequence stream in 16 MiB
    chunks: the digest of the pairs equals the reference's."""
    fx = G.fixture("scale_reads_k31_m21")
    data = G.case_input("scale_reads_k31_m21")
    stream = ctx.lex(data)
    got, _ = ctx.run(31, 21, seq=stream, n_parts=fx["n"], want_results=False, digest=True, spill=(16 << 20,))
    assert got.stats["superkmers"] == fx["reference_stderr"]["superkmers"]
    assert got.digest == fx["digest"]


def test_spill_argument_errors(ctx):
    """Spill mode is chosen before the first feed, for one sample."""
    import ctypes
    import tuna_gb300 as T
    L = T.library()
    o = ctx._opts(31, 21, 16, 1, U64_MAX, 0)
    j = ctypes.c_void_p()
    ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
    try:
        s = np.frombuffer(b"ACGT" * 100, dtype=np.uint8)
        ctx.check(L.tg_job_feed_seq(j, s.ctypes.data, s.size))
        assert L.tg_job_set_spill(j, 1 << 20, None) == 4  # TG_ERR_STATE
    finally:
        L.tg_job_end(j)
    ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
    try:
        ctx.check(L.tg_job_next_sample(j))
        assert L.tg_job_set_spill(j, 1 << 20, None) == 9  # TG_ERR_UNSUPPORTED
    finally:
        L.tg_job_end(j)
    ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
    try:
        assert L.tg_job_set_spill(j, 1 << 20, os.fsencode("/nonexistent/dir")) == 5  # TG_ERR_IO
    finally:
        L.tg_job_end(j)
