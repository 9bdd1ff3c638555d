"""FASTA/FASTQ lexing on the device (csrc/tg_lex.cu) against the oracle's
parser, which follows the reference's helicase parsers
(include/helicase_cpp/parser_fasta.hpp:233-316, parser_fastq.hpp:112-285) and is
pinned by the golden fixtures.

The device lexer counts FASTQ lines where the reference walks 64-byte blocks.
The CPU test states the lexer's rules in Python (line counting plus the two
places where the block walk departs from it) and checks them against the
oracle on fuzzed input; the GPU tests check the kernels against the oracle,
including the files the lexer hands to the host parser."""
import ctypes
import random
import re

import numpy as np
import pytest

from oracle import oracle as O

_RUN = re.compile(rb"[^ACGTacgt]+")


def runs(stream: bytes):
    return [r for r in _RUN.split(stream) if r]


def lexer_rules(data: bytes):
    """The device lexer's output for data, byte by byte, and whether it flags
    the file for the host parser."""
    out = bytearray()
    n = len(data)
    if data[:1] == b"@":
        lf_total = data.count(b"\n")
        last_na = max((i for i in range(n) if data[i:i + 1] not in (b"A", b"C", b"G", b"T", b"a", b"c", b"g", b"t")),
                      default=-1)
        drop = last_na + 1 if (lf_total % 4 == 1 and n % 64 == 0 and last_na < n - 1) else n
        line, irregular = 0, False
        for i, c in enumerate(data):
            if line % 4 == 1 and i < drop:
                out.append(c)
            if c == 10:
                if i % 64 == 63 and data[i - 1] == 10 and line % 4 == 0:
                    irregular = True
                line += 1
        return bytes(out), irregular
    state = 0  # before the first '>', 1 header, 2 sequence
    for c in data:
        if state == 0:
            if c == 62:
                out.append(10)
                state = 1
        elif state == 1:
            if c == 10:
                state = 2
        elif c == 62:
            out.append(10)
            state = 1
        elif c != 10:
            out.append(c)
    return bytes(out), False


def fuzz_case(rng: random.Random) -> bytes:
    kind = rng.random()
    if kind < 0.3:
        alph = [b"A", b"C", b"G", b"T", b"a", b"N", b"\n", b">", b"@", b"+", b"\r", b"I"]
        s = b"".join(rng.choices(alph, weights=[rng.random() for _ in alph], k=rng.randint(1, 400)))
        s = rng.choice([b"@", b">", b""]) + s
    elif kind < 0.65:
        recs = []
        for _ in range(rng.randint(1, 12)):
            L = rng.randint(0, 90)
            seq = b"".join(rng.choices([b"A", b"C", b"G", b"T", b"N", b"a"], weights=[5, 5, 5, 5, 0.3, 0.5], k=L))
            r = b"@r" + str(rng.randint(0, 99)).encode() + b"\n" + seq + b"\n+\n" + b"I" * L + b"\n"
            if rng.random() < 0.15:
                r = b"\n" + r
            if rng.random() < 0.05:
                r += b"\n"
            recs.append(r)
        s = b"".join(recs)
        if rng.random() < 0.5:
            s = s[: rng.randint(1, len(s))]
    else:
        parts = [b"junk" if rng.random() < 0.1 else b""]
        for _ in range(rng.randint(1, 8)):
            parts.append(b">h" + bytes(rng.choices(b"ACGT >x", k=rng.randint(0, 10))) + b"\n")
            for _ in range(rng.randint(0, 6)):
                line = bytes(rng.choices(b"ACGTNacgt>\r", weights=[5, 5, 5, 5, .3, 1, 1, 1, 1, .1, .1],
                                         k=rng.randint(0, 70)))
                parts.append(line + (b"\n" if rng.random() < 0.9 else b""))
        s = b"".join(parts)
        if rng.random() < 0.3:
            s = s[: rng.randint(1, len(s))]
    if s and rng.random() < 0.3 and len(s) % 64:  # lengths that are multiples of 64
        s += b"A" * (64 - len(s) % 64)
    return s or b">"


def test_lexer_rules_match_block_walk():
    rng = random.Random(5)
    flagged = 0
    for _ in range(3000):
        s = fuzz_case(rng)
        out, irregular = lexer_rules(s)
        if irregular:
            flagged += 1
            continue
        assert runs(out) == O.parse_fastx(s), s[:200]
    assert flagged < 60


def test_host_parser_matches_oracle(tmp_path):
    """The library's host parser (tgh::fastx_to_stream, the path of the FASTQ
    files the device lexer flags), driven on CPU by tests/cpp/host_parser_check.cpp
    over fuzzed files, plain and gzip: the same runs as the oracle's parser,
    including the block-walk cases the lexer hands over."""
    import gzip
    import os
    import shutil
    import subprocess

    import tuna_gb300.build as B
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = B.gpu_lib()
    exe = str(tmp_path / "host_parser_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "tuna_gb300", "csrc"),
                        "-I", os.path.join(root, "include"), os.path.join(root, "tests", "cpp", "host_parser_check.cpp"),
                        "-o", exe, "-L", os.path.dirname(lib), "-ltuna_gpu", "-Wl,-rpath," + os.path.dirname(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rng = random.Random(23)
    cases, paths = [], []
    for i in range(1500):
        s = fuzz_case(rng)
        if i % 10 == 0:  # a FASTQ record in front: the rest is read with FASTQ rules
            s = b"@r\nACGT\n+\nIIII\n" + s
        name = str(tmp_path / (f"c{i}.fq.gz" if i % 7 == 0 else f"c{i}.fa"))
        with open(name, "wb") as f:
            f.write(gzip.compress(s) if name.endswith(".gz") else s)
        cases.append(s)
        paths.append(name)
    for i in range(0, len(paths), 500):
        r = subprocess.run([exe, *paths[i:i + 500]], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
    flagged = 0
    for s, name in zip(cases, paths):
        _, irregular = lexer_rules(s)
        flagged += irregular
        with open(name + ".stream", "rb") as f:
            assert runs(f.read()) == O.parse_fastx(s), s[:200]
    assert flagged > 0  # the block-walk departures were among the cases


# ------------------------------------------------------------------ GPU

def _ctx():
    import tuna_gb300 as T
    return T.Context(0)


@pytest.mark.gpu
def test_lex_fuzz_matches_oracle():
    rng = random.Random(11)
    with _ctx() as ctx:
        for _ in range(400):
            s = fuzz_case(rng)
            assert runs(ctx.lex(s)) == O.parse_fastx(s), s[:200]


def _big_fasta(rng: random.Random, n_contigs: int, width: int) -> bytes:
    out = []
    for c in range(n_contigs):
        out.append(b">contig_" + str(c).encode() + b" some description >x\n")
        L = rng.randint(1, 200_000)
        seq = bytes(rng.choices(b"ACGTacgtN", weights=[8, 8, 8, 8, 1, 1, 1, 1, .2], k=L))
        out += [seq[i:i + width] + b"\n" for i in range(0, L, width)]
    return b"".join(out)


@pytest.mark.gpu
@pytest.mark.parametrize("width", [60, 61, 80, 16383])
def test_lex_large_fasta(width):
    rng = random.Random(width)
    fa = _big_fasta(rng, 40, width)
    with _ctx() as ctx:
        assert runs(ctx.lex(fa)) == O.parse_fastx(fa)
        cut = fa[: len(fa) - 7]  # ends inside a line
        assert runs(ctx.lex(cut)) == O.parse_fastx(cut)


@pytest.mark.gpu
@pytest.mark.parametrize("tail", ["full", "cut", "pad64"])
def test_lex_large_fastq(tail):
    from tuna_gb300 import synth
    g = synth.genome(200_000, 3, 0.45)
    fq = synth.reads_fastq(g, 20_000, (100, 250), 0.005, 0.001, 9).tobytes()
    if tail == "cut":
        fq = fq[: len(fq) - len(fq) // 3]
        fq = fq[: fq.rfind(b"\n@") + 1] + b"@last\nACGTACGTAC"  # sequence line with no LF
    elif tail == "pad64":
        fq = fq[: fq.rfind(b"\n@") + 1] + b"@last\n"
        fq += b"ACGT" * 40
        fq = fq[: len(fq) - len(fq) % 64]  # length a multiple of 64, ending on ACGT: the last run is dropped
        assert len(fq) % 64 == 0 and fq[-1:] in b"ACGT"
    with _ctx() as ctx:
        got = runs(ctx.lex(fq))
    want = O.parse_fastx(fq)
    assert got == want
    if tail == "pad64":  # the last sequence line is cut on an ACGT byte: its run is dropped
        assert fq.count(b"\n") % 4 == 1 and not want[-1].startswith(b"ACGTACGT")


def _irregular_fastq() -> bytes:
    """A FASTQ whose fourth record starts with an empty header line whose LF
    is at file offset 127 (63 mod 64)."""
    recs = b"@a\nACGTACGTAAAC\n+\nIIIIIIIIIIII\n" * 3
    pad = 127 - len(recs)  # the last quality line's LF at offset 126
    assert pad > 0
    recs = recs[:-1] + b"I" * pad + b"\n"
    s = recs + b"\n@b\nGGGGCCCCAAAATTTTGGCA\n+\nIIIIIIIIIIIIIIIIIIII\n@c\nTTTTGGGGCCCCAAAAC\n+\nIIIIIIIIIIIIIIIII\n"
    assert s[127:128] == b"\n" and s[126:127] == b"\n"
    return s


@pytest.mark.gpu
def test_lex_irregular_fastq_goes_to_host_parser():
    s = _irregular_fastq()
    _, flagged = lexer_rules(s)
    assert flagged
    want = O.parse_fastx(s)
    assert runs(lexer_rules(s)[0]) != want  # line counting alone would differ here
    with _ctx() as ctx:
        assert runs(ctx.lex(s)) == want
        res, _ = ctx.run(9, 5, fastx=s)
        assert res.stats["host_parsed_bytes"] == len(s)
    ref = O.count_fastx(s, 9, 5)
    import tuna_gb300 as T
    assert T.tsv_blob(res.keys, res.counts, 9) == O.tsv_blob(ref)


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [0, 3])
def test_feed_fastx_device(offset):
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, _ = synth.reads_workload(scale=0.01, seed=4)
    buf = torch.zeros(fq.size + 16, dtype=torch.uint8, device="cuda")
    buf[offset: offset + fq.size] = torch.from_numpy(fq).cuda()
    torch.cuda.synchronize()
    with _ctx() as ctx:
        got, _ = ctx.run(31, 21, dev_fastx=buf.data_ptr() + offset, dev_len=int(fq.size))
        assert got.stats["fastx_bytes"] == fq.size and got.stats["host_parsed_bytes"] == 0
    want = O.count_fastx(fq, 31, 21, threads=4)
    assert T.tsv_blob(got.keys, got.counts, 31) == O.tsv_blob(want)


@pytest.mark.gpu
@pytest.mark.parametrize("k,m", [(31, 23), (63, 21)])
def test_count_fastx_one_call(k, m):
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g, lens = synth.repetitive_genome(scale=0.002, seed=3)
    fa = synth.fasta(g, lens)
    L = T.library()
    W = 1 if k <= 31 else 2
    cap = int(fa.size)
    h_in = torch.from_numpy(fa).pin_memory()
    keys = torch.zeros(cap * W, dtype=torch.int64, pin_memory=True)
    cnt = torch.zeros(cap, dtype=torch.int32, pin_memory=True)
    o = T._JobOpts(k, m, 16, 1, (1 << 64) - 1, 0, 0)
    n_out = ctypes.c_uint64()
    st = T._Stats()
    with _ctx() as ctx:
        rc = L.tg_count_fastx(ctx.h, ctypes.byref(o), ctypes.c_void_p(h_in.data_ptr()), int(fa.size),
                              ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(cnt.data_ptr()), cap,
                              ctypes.byref(n_out), ctypes.byref(st))
        assert rc == 0, L.tg_last_error(ctx.h)
        assert st.fastx_bytes == fa.size and st.lex_ms > 0
    n = int(n_out.value)
    got = T.Result(keys.numpy().view(np.uint64)[: n * W].reshape(n, W), cnt.numpy().view(np.uint32)[:n], {}, k)
    want = O.count_fastx(fa, k, m, threads=4)
    assert T.tsv_blob(got.keys, got.counts, k) == O.tsv_blob(want)
