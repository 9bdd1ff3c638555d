"""Inputs of the golden fixtures. Shared by make_golden.py (which runs the
reference on them) and the tests (which regenerate them and compare).

Inline inputs are small hand-written FASTA/FASTQ files covering the edge cases
of the reference's parser and superkmer cutter; synthetic inputs come from
tuna_gb300.synth with a fixed seed and are regenerated on any host.
"""
from __future__ import annotations

import gzip
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _lines(seq: bytes, width: int = 60) -> bytes:
    return b"".join(seq[i:i + width] + b"\n" for i in range(0, len(seq), width))


def _rand_dna(n: int, seed: int) -> bytes:
    rng = np.random.default_rng(seed)
    return bytes(np.frombuffer(b"ACGT", dtype=np.uint8)[rng.integers(0, 4, n)])


def edge_fasta() -> bytes:
    """Headers, lowercase, N/IUPAC splits, a record of exactly 31 bases, a
    10 kbp poly-A (forces the 255-base record cap), '>' inside a sequence
    line, CRLF lines, empty records, text before the first header, blank
    lines and no final newline."""
    r = _rand_dna(4000, 5)
    parts = [
        b"stray text before any header ACGTACGTACGTACGTACGTACGTACGTACGTACGT\n",
        b">hdr1 ACGT in header > and more\n",
        _lines(r[:700]),
        b">lower\n", _lines(r[700:900].lower() + r[900:1000]),
        b">nsplit\n", r[1000:1030] + b"N" + r[1030:1061] + b"NN" + r[1061:1200] + b"\n",
        b">exact31\n", r[1200:1231] + b"\n",
        b">exact30\n", r[1231:1261] + b"\n",
        b">polyA\n", _lines(b"A" * 10000),
        b">polyAC\n", _lines(b"AC" * 2000 + r[1261:1400] + b"ACG" * 700),
        b">gt_in_line\n", r[1400:1500] + b">this is a header now ACGTACGT\n" + r[1500:1600] + b"\n",
        b">crlf\r\n", r[1600:1660] + b"\r\n" + r[1660:1720] + b"\r\n" + r[1720:1780] + b"\r\n",
        b">empty\n", b">\n",
        b">iupac\n", r[1780:1840] + b"RYKM" + r[1840:1900] + b"SWBDHV" + r[1900:2000] + b"\n",
        b"\n\n",
        b">blank_lines\n", r[2000:2040] + b"\n\n" + r[2040:2080] + b"\n",
        b">tabs\n", r[2080:2120] + b" \t" + r[2120:2200] + b"\n",
        b">last no newline\n", r[2200:2400],
    ]
    return b"".join(parts)


def edge_fastq() -> bytes:
    """Reads with N, lowercase, short reads, CRLF, quality lines containing
    ACGT letters, a blank line between records (malformed input whose
    handling depends on the reference's 64-byte block walk) and no final
    newline."""
    r = _rand_dna(3000, 9)
    recs = []
    pos = 0

    def rd(n):
        nonlocal pos
        s = r[pos:pos + n]
        pos += n
        return s

    recs.append(b"@r1\n" + rd(20) + b"N" + rd(60) + b"\n+\n" + b"I" * 81 + b"\n")
    recs.append(b"@r2 lower\n" + rd(40).lower() + rd(40) + b"\n+\n" + b"?" * 80 + b"\n")
    recs.append(b"@r3 short\n" + rd(10) + b"\n+\n" + b"?" * 10 + b"\n")
    recs.append(b"@r4 crlf\r\n" + rd(70) + b"\r\n+\r\n" + b"?" * 70 + b"\r\n")
    recs.append(b"@r5 acgt quality\n" + rd(64) + b"\n+\n" + b"ACGT" * 16 + b"\n")
    recs.append(b"@r6 exact\n" + rd(31) + b"\n+\n" + b"?" * 31 + b"\n")
    recs.append(b"\n")
    recs.append(b"@r7 after a blank line\n" + rd(90) + b"\n+\n" + b"?" * 90 + b"\n")
    recs.append(b"@r8\n" + rd(150) + b"\n+\n" + b"?" * 150 + b"\n")
    recs.append(b"@r9 poly\n" + b"T" * 300 + b"\n+\n" + b"?" * 300 + b"\n")
    recs.append(b"@r10 last\n" + rd(80) + b"\n+\n" + b"?" * 80)
    return b"".join(recs)


def fuzz_fastq(seed: int) -> bytes:
    """Random FASTQ-like text: valid records mixed with blank lines, N runs,
    short lines and CR, so that the 64-byte block walk is exercised at many
    alignments."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(400):
        u = rng.random()
        if u < 0.05:
            out.append(b"\n")
            continue
        L = int(rng.integers(1, 200))
        s = bytearray(_rand_dna(L, int(rng.integers(1 << 30))))
        for _ in range(int(rng.integers(0, 3))):
            s[int(rng.integers(0, L))] = ord("N")
        if rng.random() < 0.1:
            s = bytearray(bytes(s).lower())
        q = b"?" * L
        eol = b"\r\n" if rng.random() < 0.05 else b"\n"
        out.append(b"@q%d" % i + eol + bytes(s) + eol + b"+" + eol + q + b"\n")
    return b"".join(out)


def fuzz_fasta(seed: int) -> bytes:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(200):
        out.append(b">f%d %d\n" % (i, int(rng.integers(1 << 20))))
        L = int(rng.integers(0, 600))
        s = bytearray(_rand_dna(L, int(rng.integers(1 << 30))))
        for _ in range(int(rng.integers(0, 4))):
            if L:
                s[int(rng.integers(0, L))] = ord("NRYacgt"[int(rng.integers(0, 7))])
        w = int(rng.integers(10, 120))
        out.append(_lines(bytes(s), w))
        if rng.random() < 0.05:
            out.append(b"\n")
    return b"".join(out)


def synth_reads(scale: float, seed: int) -> bytes:
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=scale, seed=seed)
    return fq.tobytes()


def synth_rep_fasta(scale: float, seed: int) -> bytes:
    from tuna_gb300 import synth
    fa, _ = synth.repetitive_fasta(scale=scale, seed=seed)
    return fa.tobytes()


def synth_large_k(scale: float, seed: int) -> bytes:
    from tuna_gb300 import synth
    fq, _ = synth.large_k_reads(scale=scale, seed=seed)
    return fq.tobytes()


GENERATORS = {
    "edge_fasta": lambda s: edge_fasta(),
    "edge_fastq": lambda s: edge_fastq(),
    "fuzz_fastq": lambda s: fuzz_fastq(s["seed"]),
    "fuzz_fasta": lambda s: fuzz_fasta(s["seed"]),
    "ci_smoke": lambda s: (b">seq1\nACGTACGTACGTACGTACGTACGTACGTACGTACGT\n"
                           b">seq2\nTGCATGCATGCATGCATGCATGCATGCATGCATGCA\n"),
    "synth_reads": lambda s: synth_reads(s["scale"], s["seed"]),
    "synth_rep_fasta": lambda s: synth_rep_fasta(s["scale"], s["seed"]),
    "synth_large_k": lambda s: synth_large_k(s["scale"], s["seed"]),
}


def _inline(gen: str, **kw) -> dict:
    return {"kind": "inline", "gen": gen, **kw}


def _synth(gen: str, **kw) -> dict:
    return {"kind": "synth", "gen": gen, **kw}


CASES = [
    dict(name="ci_smoke_k31", k=31, m=21, n=4, source=_inline("ci_smoke"), store_full=True),
    dict(name="edge_fasta_k31", k=31, m=21, source=_inline("edge_fasta"), store_full=True, parts=True),
    dict(name="edge_fasta_k15", k=15, m=9, source=_inline("edge_fasta"), store_full=True),
    dict(name="edge_fasta_k5", k=5, m=3, n=4, source=_inline("edge_fasta"), store_full=True),
    dict(name="edge_fasta_k63", k=63, m=21, source=_inline("edge_fasta"), store_full=True, parts=True),
    dict(name="edge_fastq_k31", k=31, m=21, source=_inline("edge_fastq"), store_full=True),
    dict(name="edge_fastq_k9", k=9, m=5, source=_inline("edge_fastq"), store_full=True),
    dict(name="fuzz_fastq_k15", k=15, m=9, source=_inline("fuzz_fastq", seed=3), store_full=True),
    dict(name="fuzz_fastq_k31", k=31, m=21, source=_inline("fuzz_fastq", seed=4), store_full=True),
    dict(name="fuzz_fasta_k21", k=21, m=17, source=_inline("fuzz_fasta", seed=5), store_full=True),
    dict(name="fuzz_fasta_k33", k=33, m=21, source=_inline("fuzz_fasta", seed=6), store_full=True),
    dict(name="edge_fasta_k139", k=139, m=21, source=_inline("edge_fasta"), store_full=True),
    dict(name="reads_k31_m21", k=31, m=21, n=64, source=_synth("synth_reads", scale=0.01, seed=1),
         parts=True),
    dict(name="reads_k31_m21_ci2", k=31, m=21, n=32, ci=2, cx=40,
         source=_synth("synth_reads", scale=0.01, seed=1)),
    dict(name="reads_k25_m21", k=25, m=21, source=_synth("synth_reads", scale=0.01, seed=2)),
    dict(name="reads_k21_m17", k=21, m=17, source=_synth("synth_reads", scale=0.01, seed=3)),
    dict(name="rep_fasta_k31_m23", k=31, m=23, n=256, source=_synth("synth_rep_fasta", scale=0.001, seed=7),
         parts=True),
    dict(name="large_k63_m21", k=63, m=21, n=64, ci=2, cx=10000,
         source=_synth("synth_large_k", scale=0.005, seed=11), parts=True),
]


# Digest fixtures at the benchmarked sizes. The reference's TSV output for these
# inputs (billions of lines at full size) is recorded as the order-independent
# digest of oracle/tuna_digest.h (the one tg_job_result_digest computes), with
# the line count and the superkmers: value. Inputs are regenerated from their
# seed; their sha256 pins them.
#   scale_reads_*      the small read set at its full size (138 Mbp of reads)
#   scale_rep_fasta_*  the repetitive assembly at 1/10 (310 Mbp)
#   scale_large_k63_*  the k=63 read set at 1/10 (300 Mbp of reads), ci/cx
#   bench_*            the bench's full-size workloads (3.1 Gbp assembly,
#                      3 Gbp k=63 read set), checked by bench.py
SCALE_CASES = [
    dict(name="scale_reads_k31_m21", k=31, m=21, n=64, source=_synth("synth_reads", scale=1.0, seed=1)),
    dict(name="scale_rep_fasta_k31_m23", k=31, m=23, n=4096,
         source=_synth("synth_rep_fasta", scale=0.1, seed=7)),
    dict(name="scale_large_k63_m21", k=63, m=21, n=64, ci=2, cx=10000,
         source=_synth("synth_large_k", scale=0.1, seed=11)),
    dict(name="bench_rep_fasta_k31_m23", k=31, m=23, n=4096,
         source=_synth("synth_rep_fasta", scale=1.0, seed=7)),
    dict(name="bench_large_k63_m21", k=63, m=21, n=64, ci=2, cx=10000,
         source=_synth("synth_large_k", scale=1.0, seed=11)),
]


def input_bytes(case: dict) -> bytes:
    src = case["source"]
    return GENERATORS[src["gen"]](src)


def load_input(case: dict) -> bytes:
    """The input bytes of a case: the committed copy for inline inputs when
    present, else regenerated."""
    p = os.path.join(HERE, case["name"] + ".in.gz")
    if case["source"]["kind"] == "inline" and os.path.exists(p):
        with gzip.open(p, "rb") as f:
            return f.read()
    return input_bytes(case)
