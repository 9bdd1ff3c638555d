"""The CPU oracle against the reference's own outputs (tests/golden/).

Every GPU parity test compares against the oracle, so it is pinned here
first: same sorted (k-mer, count) lines, same superkmer count, and the same
Phase 1 partition contents (record multisets) as the reference binaries.
"""
import pytest

from oracle import oracle as O
from tests import golden_util as G


@pytest.mark.parametrize("name", G.CASE_NAMES)
def test_counts_match_reference(name):
    fx = G.fixture(name)
    data = G.case_input(name)
    cx = fx["cx"] if fx["cx"] is not None else (1 << 64) - 1
    res = O.count_fastx(data, fx["k"], fx["m"], n_parts=fx["n"], ci=fx["ci"], cx=cx, threads=4)
    blob = O.tsv_blob(res)
    full = G.full_tsv(name)
    if full is not None and blob != full:
        got, want = set(blob.decode().splitlines()), set(full.decode().splitlines())
        pytest.fail(f"{name}: {len(got - want)} extra, {len(want - got)} missing; "
                    f"e.g. extra {sorted(got - want)[:3]} missing {sorted(want - got)[:3]}")
    assert len(res) == fx["lines"]
    assert G.sha(blob) == fx["tsv_sha256"]
    assert res.stats["n_superkmers"] == fx["reference_stderr"]["superkmers"]


@pytest.mark.parametrize("name", [n for n in G.CASE_NAMES if G.parts_fixture(n)])
def test_partitions_match_reference(name):
    pj = G.parts_fixture(name)
    data = G.case_input(name)
    stream = O.fastx_to_stream(data)
    parts = O.partition_stream(stream, pj["k"], pj["m"], pj["n"], threads=2)
    assert len(parts) == len(pj["partitions"])
    for p, (blob, want) in enumerate(zip(parts, pj["partitions"])):
        recs = O.split_records(blob, pj["k"], pj["m"])
        assert len(recs) == want["records"], f"partition {p}"
        assert len(blob) == want["bytes"], f"partition {p}"
        assert G.record_multiset_sha(recs) == want["sha256"], f"partition {p}"


def test_nthash_known_values():
    # canonical hash is strand-symmetric and equals fwd ^ rev of the seeds
    s = b"ACGTACGTACGTACGTACGTA"
    rc = bytes({65: 84, 67: 71, 71: 67, 84: 65}[c] for c in reversed(s))
    assert O.nthash(s) == O.nthash(rc)
    # m = 1: fwd = FWD[b], rev = REV[b] = FWD[b ^ 2] (nt_hash.hpp:26-40)
    fwd = {b"A": 0x3c8bfbb395c60474, b"C": 0x3193c18562a02b4c,
           b"T": 0x295549f54be24456, b"G": 0x20323ed082572324}
    assert O.nthash(b"A") == fwd[b"A"] ^ fwd[b"T"]
    assert O.nthash(b"C") == fwd[b"C"] ^ fwd[b"G"]


def test_empty_input_raises():
    with pytest.raises(RuntimeError, match="Empty file"):
        O.count_fastx(b"", 31, 21)
