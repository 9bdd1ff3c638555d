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
