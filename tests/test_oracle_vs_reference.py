"""The oracle against the reference itself on fresh seeded inputs, beyond the
committed fixtures: the reference CLI built from its own sources
(oracle/build_ref.sh, binaries in oracle/_ref/, present only where the
reference sources are) and the oracle give the same sorted (k-mer, count)
lines and the same superkmers: count on random FASTA and FASTQ, with and
without -ci/-cx. Skipped where the reference binaries are absent."""
import os
import random
import subprocess

import pytest

from oracle import oracle as O
from tests.test_oracle_bruteforce import _fasta, _fastq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
PAIRS = [(5, 3), (9, 5), (15, 9), (21, 17), (25, 21), (31, 21), (31, 23), (33, 21), (63, 21)]


def _bin(k, m):
    return os.path.join(REF, f"tuna_k{k}_m{m}")


def _run_reference(k, m, data: bytes, tmp, ci=1, cx=None):
    inp = os.path.join(tmp, "in.fq" if data[:1] == b"@" else "in.fa")
    with open(inp, "wb") as f:
        f.write(data)
    out = os.path.join(tmp, "out.tsv")
    cmd = [_bin(k, m), "-k", str(k), "-m", str(m), "-n", "16", "-t", "2", "-hp"]
    if ci != 1:
        cmd += ["-ci", str(ci)]
    if cx is not None:
        cmd += ["-cx", str(cx)]
    cmd += ["-w", os.path.join(tmp, "wd"), inp, out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    with open(out, "rb") as f:
        lines = b"".join(sorted(f.read().splitlines(keepends=True)))
    sk = [int(ln.split(":", 1)[1]) for ln in r.stderr.splitlines() if ln.startswith("superkmers:")]
    return lines, sk[0] if sk else None


@pytest.mark.parametrize("k,m", PAIRS)
def test_oracle_equals_reference_binary(tmp_path, k, m):
    if not os.path.exists(_bin(k, m)):
        pytest.skip("reference binary not built here")
    rng = random.Random(7919 * k + m)
    for i in range(6):
        data = _fasta(rng, rng.randint(5, 60)) if i % 2 == 0 else _fastq(rng, rng.randint(20, 200))
        data = data + data[: len(data) // 3].rsplit(b"\n", 1)[0] + b"\n" if i % 3 == 0 else data
        ci, cx = (2, rng.randint(2, 6)) if i == 5 else (1, None)
        want, sk = _run_reference(k, m, data, str(tmp_path), ci, cx)
        got = O.count_fastx(data, k, m, ci=ci, cx=cx if cx is not None else (1 << 64) - 1, threads=2)
        assert O.tsv_blob(got) == want, (k, m, i)
        assert sk is None or got.stats["n_superkmers"] == sk, (k, m, i)
