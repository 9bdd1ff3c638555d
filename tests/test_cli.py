"""The `tuna` command line (tuna_gb300/csrc/cli/tuna_main.cpp) against the
reference CLI: argument errors (text and exit code, against the reference
binary built from its sources when it is present), output bytes, the stderr
keys, KFF output and the -tp -kt partition files."""
import hashlib
import os
import struct
import subprocess

import pytest

from tests import golden_util as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "tuna_k31_m21")


@pytest.fixture(scope="module")
def cli():
    import tuna_gb300.build as B
    return B.cli()


BAD_ARGS = [
    [],
    ["-k"],
    ["-k", "300", "a.fa", "out.tsv"],
    ["-k", "1", "a.fa", "out.tsv"],
    ["-m", "40", "a.fa", "out.tsv"],
    ["-m", "31", "a.fa", "out.tsv"],
    ["-m", "0", "a.fa", "out.tsv"],
    ["-q", "a.fa", "out.tsv"],
    ["-t", "0", "a.fa", "out.tsv"],
    ["-k", "x31", "a.fa", "out.tsv"],
    ["-n", "99999999999", "a.fa", "out.tsv"],
    ["only_one_arg"],
    ["@/nonexistent/list.txt", "out.tsv"],
    ["-k", "31x", "a.fa", "out.tsv"],
    ["-k", "", "a.fa", "out.tsv"],
    ["-ci", "99999999999999999999999", "a.fa", "out.tsv"],
    ["-ci", "4294967296", "a.fa", "out.tsv"],
    ["-ram", "x", "a.fa", "out.tsv"],
    ["-ram", "17179869184", "a.fa", "out.tsv"],
    ["-w"],
    ["-t", "-1", "a.fa", "out.tsv"],
    ["-m", "31", "-k", "31", "a.fa", "out.tsv"],
    ["-k", "40", "-m", "20", "-t", "0", "-h", "a.fa", "out.tsv"],
    ["-x", "-k", "31"],
    ["a.fa", "-k"],
    ["-h"],
]


def _err_line(stderr: str) -> str:
    for ln in stderr.splitlines():
        if ln.startswith("tuna: error:"):
            return ln
    return ""


@pytest.mark.parametrize("args", BAD_ARGS, ids=[" ".join(a) or "none" for a in BAD_ARGS])
def test_argument_errors(cli, args, tmp_path):
    """Exit code 1 and a "tuna: error:" line (or the usage text) before any
    device work; the same line as the reference CLI when its binary is here."""
    r = subprocess.run([cli, *args], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1
    assert _err_line(r.stderr) or "Usage" in r.stderr or "usage" in r.stderr
    if os.path.exists(REF_BIN):
        ref = subprocess.run([REF_BIN, *args], capture_output=True, text=True, cwd=tmp_path)
        assert ref.returncode == r.returncode
        assert _err_line(ref.stderr) == _err_line(r.stderr)


HEADER_ARGS = [
    ["-k", " 25", "-m", "+13"],
    ["-cx", "-1"],
    ["-ci", "3", "-cx", "100", "-t", "2"],
    ["-k", "33", "-m", "17", "-n", "0"],
]


@pytest.mark.parametrize("args", HEADER_ARGS, ids=[" ".join(a) for a in HEADER_ARGS])
def test_accepted_forms_header(cli, tmp_path, args):
    """Integer forms std::stoull accepts (blanks, signs, wrap-around of "-1")
    are accepted alike: the header line equals the reference binary's."""
    (tmp_path / "a.fa").write_bytes(b">s\nACGTACGTTGCAACGTAGCTAGCTAGGATCCATGCATGCA\n")
    r = subprocess.run([cli, *args, "a.fa", "out.tsv"], capture_output=True, text=True, cwd=tmp_path)
    head = [ln for ln in r.stderr.splitlines() if ln.startswith("tuna  k=")]
    assert head, r.stderr
    if os.path.exists(REF_BIN) and "-k" not in args:
        ref = subprocess.run([REF_BIN, *args, "a.fa", "ref.tsv"], capture_output=True, text=True, cwd=tmp_path)
        assert [ln for ln in ref.stderr.splitlines() if ln.startswith("tuna  k=")] == head


def _header_n(stderr: str) -> str:
    for ln in stderr.splitlines():
        if ln.startswith("tuna  k="):
            return [f for f in ln.split() if f.startswith("n=")][0]
    return ""


@pytest.mark.parametrize("n,want", [("1", "n=1"), ("3", "n=4"), ("1000", "n=1024"), ("4096", "n=4096"),
                                    ("5000", "n=8192"), ("2147483648", "n=2147483648"),
                                    ("2147483649", "n=0")])
def test_partition_count_rounding(cli, tmp_path, n, want):
    """-n is rounded up to a power of two as the reference's main does (the
    header line is printed before any device work); against the reference
    binary for the counts it can run quickly."""
    (tmp_path / "a.fa").write_bytes(b">s\nACGTACGTTGCAACGTAGCTAGCTAGGATCCATGCATGCA\n")
    r = subprocess.run([cli, "-n", n, "a.fa", "out.tsv"], capture_output=True, text=True, cwd=tmp_path)
    assert _header_n(r.stderr) == want
    if os.path.exists(REF_BIN) and int(n) <= 8192:
        ref = subprocess.run([REF_BIN, "-n", n, "a.fa", "ref.tsv"], capture_output=True, text=True, cwd=tmp_path)
        assert _header_n(ref.stderr) == want


def _write_case(tmp_path, name):
    data = G.case_input(name)
    path = tmp_path / ("in.fq" if data[:1] == b"@" else "in.fa")
    path.write_bytes(data)
    return path


def _stderr_keys(text: str) -> dict:
    out = {}
    for ln in text.splitlines():
        if ": " in ln and not ln.startswith("tuna"):
            key, val = ln.split(": ", 1)
            out[key.strip()] = val.strip()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["edge_fasta_k31", "edge_fastq_k31", "fuzz_fasta_k33", "reads_k31_m21_ci2"])
def test_tsv_output_and_stderr(cli, tmp_path, name):
    fx = G.fixture(name)
    inp = _write_case(tmp_path, name)
    out = tmp_path / "out.tsv"
    args = [cli, "-k", str(fx["k"]), "-m", str(fx["m"]), "-n", str(fx["n"]), "-ci", str(fx["ci"])]
    if fx["cx"] is not None:
        args += ["-cx", str(fx["cx"])]
    r = subprocess.run(args + ["-hp", str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = sorted(out.read_bytes().split(b"\n")[:-1])
    blob = b"\n".join(lines) + b"\n" if lines else b""
    assert hashlib.sha256(blob).hexdigest() == fx["tsv_sha256"]
    keys = _stderr_keys(r.stderr)
    for key in ("phase1", "phase2", "superkmers", "n_parts", "unique_kmers"):
        assert key in keys, r.stderr
    want = fx["reference_stderr"]
    assert int(keys["superkmers"]) == want["superkmers"]
    assert int(keys["n_parts"]) == want["n_parts"]
    assert int(keys["unique_kmers"]) == want["unique_kmers"]
    assert keys["phase1"].endswith("s") and keys["phase2"].endswith("s")


def _read_kff(blob: bytes, k: int):
    """(label, count) pairs of the raw sections of a KFF file written with the
    reference's settings (encoding A0 C1 G2 T3, max = 1, data_size = 4): each
    block is the k-mer's bases, 2 bits each from the most significant end, then
    the count as a big-endian u32."""
    assert blob[:3] == b"KFF" and blob[-3:] == b"KFF"
    pos = 3 + 2 + 1 + 1 + 1  # magic, version, encoding, uniqueness, canonicity
    (free_len,) = struct.unpack(">I", blob[pos:pos + 4])
    pos += 4 + free_len
    nbytes = (k + 3) // 4
    pairs = []
    while pos < len(blob) - 3:
        kind = blob[pos:pos + 1]
        pos += 1
        if kind == b"v":
            (nv,) = struct.unpack(">Q", blob[pos:pos + 8])
            pos += 8
            for _ in range(nv):
                end = blob.index(b"\0", pos)
                pos = end + 1 + 8
        elif kind == b"r":
            (nb,) = struct.unpack(">Q", blob[pos:pos + 8])
            pos += 8
            for _ in range(nb):  # max = 1: a block is one k-mer and its count
                seq = blob[pos:pos + nbytes]
                pos += nbytes
                (cnt,) = struct.unpack(">I", blob[pos:pos + 4])
                pos += 4
                bits = int.from_bytes(seq, "big") >> (2 * (4 * nbytes - k))
                lab = "".join("ACGT"[(bits >> (2 * (k - 1 - i))) & 3] for i in range(k))
                pairs.append((lab, cnt))
        elif kind in (b"i",):
            break
        else:
            raise AssertionError(f"unknown KFF section {kind!r} at {pos - 1}")
    return pairs


@pytest.mark.gpu
def test_kff_output(cli, tmp_path):
    name = "edge_fasta_k31"
    fx = G.fixture(name)
    inp = _write_case(tmp_path, name)
    out = tmp_path / "out.kff"
    r = subprocess.run([cli, "-k", "31", "-m", "21", "-hp", str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pairs = _read_kff(out.read_bytes(), 31)
    lines = sorted(f"{a}\t{c}".encode() for a, c in pairs)
    blob = b"\n".join(lines) + b"\n"
    assert hashlib.sha256(blob).hexdigest() == fx["tsv_sha256"]


@pytest.mark.gpu
def test_partition_files(cli, tmp_path):
    from oracle.oracle import split_records
    name = "edge_fasta_k31"
    pj = G.parts_fixture(name)
    inp = _write_case(tmp_path, name)
    wd = tmp_path / "work"
    r = subprocess.run([cli, "-k", str(pj["k"]), "-m", str(pj["m"]), "-n", str(pj["n"]), "-tp", "-kt", "-w", str(wd),
                        "-hp", str(inp), str(tmp_path / "out.tsv")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for p, want in enumerate(pj["partitions"]):
        blob = (wd / f"hash_{p}.superkmers").read_bytes()
        recs = split_records(blob, pj["k"], pj["m"])
        assert len(recs) == want["records"], f"partition {p}"
        assert len(blob) == want["bytes"], f"partition {p}"
        assert G.record_multiset_sha(recs) == want["sha256"], f"partition {p}"


@pytest.mark.gpu
def test_empty_input(cli, tmp_path):
    empty = tmp_path / "empty.fa"
    empty.write_bytes(b"")
    r = subprocess.run([cli, "-hp", str(empty), str(tmp_path / "o.tsv")], capture_output=True, text=True)
    assert r.returncode == 1
    assert "tuna: error:" in r.stderr and "Empty file" in r.stderr
