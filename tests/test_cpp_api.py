"""The C++ API (include/tuna/tuna.hpp), used as a reference user would use the
reference's tuna.hpp: count_to, count_to_raw and count with ASCII or binary
callbacks, checked against the golden fixtures (sorted TSV hash), plus its
exceptions (empty file list, missing file)."""
import hashlib
import os
import subprocess

import pytest

from tests import golden_util as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "api_check.cpp")
INC = os.path.join(ROOT, "include")


def test_header_compiles():
    """No GPU needed: the header and a program using every entry point compile."""
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", INC, SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.fixture(scope="module")
def api_bin(tmp_path_factory):
    import tuna_gb300.build as B
    lib = B.gpu_lib()
    out = str(tmp_path_factory.mktemp("cpp") / "api_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", INC, SRC, "-o", out, "-L", os.path.dirname(lib),
                        "-ltuna_gpu", "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


CASES = ["edge_fasta_k31", "edge_fastq_k31", "fuzz_fasta_k21", "fuzz_fasta_k33", "edge_fasta_k63",
         "edge_fasta_k5", "reads_k31_m21_ci2", "reads_k25_m21"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("mode", ["count_to", "raw", "cb_ascii", "cb_binary"])
def test_api_matches_reference(api_bin, tmp_path, name, mode):
    fx = G.fixture(name)
    data = G.case_input(name)
    suffix = ".fq" if data[:1] == b"@" else ".fa"
    path = tmp_path / ("in" + suffix)
    path.write_bytes(data)
    cx = fx["cx"] if fx["cx"] is not None else 0xFFFFFFFF
    r = subprocess.run([api_bin, str(fx["k"]), str(fx["m"]), mode, str(fx["ci"]), str(cx), str(path)],
                       capture_output=True)
    assert r.returncode == 0, r.stderr.decode()
    lines = sorted(r.stdout.split(b"\n")[:-1]) if r.stdout else []
    blob = b"\n".join(lines) + b"\n" if lines else b""
    assert len(lines) == fx["lines"]
    assert hashlib.sha256(blob).hexdigest() == fx["tsv_sha256"]


@pytest.mark.gpu
def test_api_errors(api_bin, tmp_path):
    r = subprocess.run([api_bin, "31", "21", "count_to", "1", "4294967295"], capture_output=True, text=True)
    assert r.returncode == 3 and "no input files" in r.stderr
    r = subprocess.run([api_bin, "31", "21", "count_to", "1", "4294967295", str(tmp_path / "missing.fa")],
                       capture_output=True, text=True)
    assert r.returncode == 4, r.stderr
    empty = tmp_path / "empty.fa"
    empty.write_bytes(b"")
    r = subprocess.run([api_bin, "31", "21", "count_to", "1", "4294967295", str(empty)], capture_output=True,
                       text=True)
    assert r.returncode == 4 and "Empty file" in r.stderr


@pytest.mark.parametrize("k", [5, 31, 32, 63])
def test_kmer_members(tmp_path, k):
    """tuna::Kmer<k> members (no device): construction from a label (any case),
    the label, reverse complement, canonical form, KFF bytes, word layout,
    order and first/last base, against a Python restatement."""
    import random
    exe = str(tmp_path / "kmer_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "kmer_check.cpp"), "-o", exe], check=True)
    rng = random.Random(k)
    labels = ["".join(rng.choice("ACGTacgt") for _ in range(k)) for _ in range(200)] + ["A" * k, "T" * k]
    r = subprocess.run([exe, str(k)], input="\n".join(labels) + "\n", capture_output=True, text=True, check=True)
    code = {"A": 0, "C": 1, "G": 2, "T": 3}
    prev = None
    for lab, out in zip(labels, r.stdout.splitlines()):
        up = lab.upper()
        rc = "".join("TGCA"["ACGT".index(c)] for c in reversed(up))
        v = 0
        for c in up:
            v = (v << 2) | code[c]
        nw = (k + 31) // 32
        words = ",".join(f"{(v >> (64 * w)) & ((1 << 64) - 1):016x}" for w in range(nw))
        packed = bytearray((k + 3) // 4)
        for i, c in enumerate(up):
            packed[i >> 2] |= code[c] << (6 - 2 * (i & 3))
        cmp = 0 if prev is None else (up > prev) - (up < prev)
        want = f"{up} {rc} {min(up, rc)} {packed.hex()} {words} {cmp} {code[up[0]]}{code[up[-1]]}"
        assert out == want, (lab, out, want)
        prev = up
