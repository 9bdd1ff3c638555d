"""The oracle against a brute-force counter written from the definitions alone.

The counter below knows nothing of ntHash, minimizers, superkmers or
partitions: it splits FASTA/FASTQ into maximal [ACGTacgt] runs by the
reference's rules (a FASTA '>' line is a header, line feeds join sequence
lines, any other byte ends a run; FASTQ is four lines per record and only the
sequence line counts), takes every k-mer of every run, keeps the smaller of it
and its reverse complement (A < C < G < T) and counts. The reference's counts
were found equal to such a counter in the survey's probe, so this pins the
oracle (and the reference-pinned fixtures) independently of how either cuts
records, for k on both sides of every key-width boundary.
"""
import random
from collections import Counter

import pytest

from oracle import oracle as O

_COMP = bytes.maketrans(b"ACGT", b"TGCA")


def _runs(data: bytes):
    seq = bytearray()
    if data[:1] == b"@":
        for i, line in enumerate(data.split(b"\n")):
            if i % 4 == 1:
                seq += line + b"\x00"
    else:
        in_header = False
        for line in data.split(b"\n"):
            if line.startswith(b">"):
                seq += b"\x00"
                in_header = True
                continue
            if in_header or line:
                in_header = False
                seq += line
    run = bytearray()
    for c in bytes(seq):
        if chr(c) in "ACGTacgt":
            run.append(c)
        else:
            if run:
                yield bytes(run).upper()
            run = bytearray()
    if run:
        yield bytes(run).upper()


def brute_force_tsv(data: bytes, k: int, ci: int = 1, cx: int = (1 << 64) - 1) -> bytes:
    counts = Counter()
    for r in _runs(data):
        for i in range(len(r) - k + 1):
            f = r[i:i + k]
            rc = f.translate(_COMP)[::-1]
            counts[min(f, rc)] += 1
    lines = sorted(b"%s\t%d\n" % (km, c) for km, c in counts.items() if ci <= c <= cx)
    return b"".join(lines)


def _fasta(rng: random.Random, n_rec: int) -> bytes:
    out = []
    for i in range(n_rec):
        body = "".join(rng.choice("ACGTACGTACGTacgtNRY") for _ in range(rng.randint(0, 400)))
        width = rng.choice([60, 70, 7, 1000])
        lines = [body[j:j + width] for j in range(0, len(body), width)] or [""]
        eol = rng.choice(["\n", "\r\n"])
        out.append(f">rec{i} some description{eol}" + eol.join(lines) + eol)
    return "".join(out).encode()


def _fastq(rng: random.Random, n_rec: int) -> bytes:
    out = []
    for i in range(n_rec):
        s = "".join(rng.choice("ACGTACGTACGTacgN") for _ in range(rng.randint(1, 200)))
        out.append(f"@read{i}\n{s}\n+\n{'I' * len(s)}\n")
    return "".join(out).encode()


@pytest.mark.parametrize("k,m", [(2, 1), (5, 3), (21, 17), (31, 21), (32, 21), (33, 21), (63, 21),
                                 (64, 21), (139, 21)])
@pytest.mark.parametrize("kind", ["fasta", "fastq"])
def test_oracle_equals_brute_force(k, m, kind):
    rng = random.Random(1000 * k + (kind == "fastq"))
    data = _fasta(rng, 40) if kind == "fasta" else _fastq(rng, 120)
    # repeats, so that counts above 1 occur
    data = data + data.replace(b">rec", b">copy").replace(b"@read", b"@copy")
    assert O.tsv_blob(O.count_fastx(data, k, m, threads=2)) == brute_force_tsv(data, k)


@pytest.mark.parametrize("ci,cx", [(2, (1 << 64) - 1), (1, 1), (2, 3)])
def test_oracle_filter_equals_brute_force(ci, cx):
    rng = random.Random(7)
    data = _fastq(rng, 200)
    data = data + data[: len(data) // 2].rsplit(b"\n@", 1)[0] + b"\n"
    assert O.tsv_blob(O.count_fastx(data, 25, 21, ci=ci, cx=cx)) == brute_force_tsv(data, 25, ci, cx)
