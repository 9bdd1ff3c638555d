"""Generate the golden fixtures of tests/golden/ by running the reference.

The reference tuna CLI is compiled from its own sources by oracle/build_ref.sh
(one binary per (k, m) in oracle/_ref/). This script runs those binaries on
seeded inputs and records what they print:

  <case>.json        parameters, sha256 of the input bytes, line count and
                     sha256 of the sorted TSV output, the superkmers /
                     unique_kmers lines of stderr; for small cases the sorted
                     TSV itself (<case>.tsv.gz) and the input (<case>.in.gz)
  <case>.parts.json  Phase 1 partition contents: per partition, the sha256 of
                     its sorted record list (records in the reference's
                     superkmer file layout, hex) and the record count

Phase 1 partition files only exist when the reference takes its disk pipeline
(estimated 2 x input size >= 60% of the -ram budget, src/pipeline.hpp:77-89).
The input is therefore padded with zero bytes to 330 MB (a sparse file; zero
bytes are non-ACGT and produce nothing) and run with -ram 1 -tp -kt -w <dir>.

Inputs made by tuna_gb300.synth are regenerated bit-identically from their
seed on any host, so only their sha256 is stored.

Scale cases (cases.SCALE_CASES, --scale): inputs of up to 3.1 Gbp whose TSV
output is too large to keep. The reference writes its TSV to standard output,
which oracle/tsv_digest reads: <case>.json then holds the digest (pairs, count
sum, h1, h2), the line count and the superkmers: value.

Usage: python tests/golden/make_golden.py [--scale [NAME ...]]   (needs
oracle/_ref/, i.e. the reference sources: TUNA_REFERENCE names their root,
else a `reference` directory beside the repository)
"""
from __future__ import annotations

import base64
import gzip
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden import cases as C  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def reference_root() -> str:
    """Root of the reference sources: $TUNA_REFERENCE, else a `reference`
    directory beside the repository."""
    env = os.environ.get("TUNA_REFERENCE")
    if env:
        return env
    return os.path.join(os.path.dirname(ROOT), "reference")


def ref_bin(k: int, m: int) -> str:
    p = os.path.join(REF, f"tuna_k{k}_m{m}")
    if not os.path.exists(p):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), reference_root(), f"{k}:{m}"])
    return p


def run_ref(case: dict, data: bytes, tmp: str):
    suffix = ".fq" if data[:1] == b"@" else ".fa"
    inp = os.path.join(tmp, case["name"] + suffix)
    with open(inp, "wb") as f:
        f.write(data)
    out = os.path.join(tmp, case["name"] + ".tsv")
    cmd = [ref_bin(case["k"], case["m"]), "-k", str(case["k"]), "-m", str(case["m"]),
           "-n", str(case.get("n", 16)), "-t", "4", "-hp"]
    if case.get("ci", 1) != 1:
        cmd += ["-ci", str(case["ci"])]
    if case.get("cx") is not None:
        cmd += ["-cx", str(case["cx"])]
    cmd += ["-w", os.path.join(tmp, "wd_" + case["name"]), inp, out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{case['name']}: reference failed: {r.stderr}")
    with open(out, "rb") as f:
        lines = sorted(f.read().decode().splitlines())
    stats = {}
    for ln in r.stderr.splitlines():
        if ":" in ln:
            key, _, val = ln.partition(":")
            if key in ("superkmers", "unique_kmers", "n_parts"):
                stats[key] = int(val.strip())
    return lines, stats


def run_ref_parts(case: dict, data: bytes, tmp: str):
    suffix = ".fq" if data[:1] == b"@" else ".fa"
    inp = os.path.join(tmp, case["name"] + "_pad" + suffix)
    with open(inp, "wb") as f:
        f.write(data)
        f.truncate(330 << 20)
    wd = os.path.join(tmp, "parts_" + case["name"])
    os.makedirs(wd, exist_ok=True)
    n = case.get("n", 16)
    cmd = [ref_bin(case["k"], case["m"]), "-k", str(case["k"]), "-m", str(case["m"]), "-n", str(n),
           "-t", "1", "-hp", "-ram", "1", "-tp", "-kt", "-w", wd, inp, os.path.join(tmp, "unused.tsv")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{case['name']}: reference phase 1 failed: {r.stderr}")
    parts = []
    for p in range(n):
        with open(os.path.join(wd, f"hash_{p}.superkmers"), "rb") as f:
            parts.append(f.read())
    shutil.rmtree(wd, ignore_errors=True)
    os.remove(inp)
    return parts


def _write_gz(path: str, data: bytes) -> None:
    with open(path, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as f:
        f.write(data)


def run_ref_digest(case: dict, data: bytes, tmp: str) -> dict:
    """The reference on a large input, its TSV piped through oracle/tsv_digest."""
    from oracle import oracle as O
    O.build()
    suffix = ".fq" if data[:1] == b"@" else ".fa"
    inp = os.path.join(tmp, case["name"] + suffix)
    with open(inp, "wb") as f:
        f.write(data)
    cmd = [ref_bin(case["k"], case["m"]), "-k", str(case["k"]), "-m", str(case["m"]),
           "-n", str(case.get("n", 16)), "-t", str(os.cpu_count() or 1), "-hp"]
    if case.get("ci", 1) != 1:
        cmd += ["-ci", str(case["ci"])]
    if case.get("cx") is not None:
        cmd += ["-cx", str(case["cx"])]
    cmd += ["-w", os.path.join(tmp, "wd_" + case["name"]), inp, "/dev/stdout"]
    err_path = os.path.join(tmp, case["name"] + ".err")
    with open(err_path, "w") as err:
        ref = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=err)
        dg = subprocess.run([O.TSV_DIGEST_BIN], stdin=ref.stdout, capture_output=True)
        ref.stdout.close()
        rc = ref.wait()
    os.remove(inp)
    with open(err_path) as f:
        stderr = f.read()
    if rc != 0 or dg.returncode != 0:
        raise RuntimeError(f"{case['name']}: reference rc {rc}, digest rc {dg.returncode}: {stderr} "
                           f"{dg.stderr.decode(errors='replace')}")
    d = json.loads(dg.stdout)
    d.pop("k", None)
    stats = {}
    for ln in stderr.splitlines():
        if ":" in ln:
            key, _, val = ln.partition(":")
            if key in ("superkmers", "unique_kmers", "n_parts"):
                stats[key] = int(val.strip())
    return {"digest": d, "reference_stderr": stats}


def main_scale(names) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        for case in C.SCALE_CASES:
            if names and case["name"] not in names:
                continue
            data = C.input_bytes(case)
            r = run_ref_digest(case, data, tmp)
            fx = {
                "name": case["name"], "k": case["k"], "m": case["m"], "n": case.get("n", 16),
                "ci": case.get("ci", 1), "cx": case.get("cx"),
                "source": case["source"], "input_bytes": len(data),
                "input_sha256": hashlib.sha256(data).hexdigest(),
                "lines": r["digest"]["pairs"], "digest": r["digest"],
                "reference_stderr": r["reference_stderr"],
            }
            with open(os.path.join(HERE, case["name"] + ".json"), "w") as f:
                json.dump(fx, f, indent=1, sort_keys=True)
            print(f"{case['name']}: {fx['lines']} lines {fx['reference_stderr']}", flush=True)


def main() -> None:
    if "--scale" in sys.argv:
        main_scale([a for a in sys.argv[1:] if a != "--scale"])
        return
    out_dir = HERE
    with tempfile.TemporaryDirectory() as tmp:
        for case in C.CASES:
            data = C.input_bytes(case)
            lines, stats = run_ref(case, data, tmp)
            blob = "".join(l + "\n" for l in lines).encode()
            fx = {
                "name": case["name"], "k": case["k"], "m": case["m"], "n": case.get("n", 16),
                "ci": case.get("ci", 1), "cx": case.get("cx"),
                "source": case["source"], "input_bytes": len(data),
                "input_sha256": hashlib.sha256(data).hexdigest(),
                "lines": len(lines), "tsv_sha256": hashlib.sha256(blob).hexdigest(),
                "reference_stderr": stats,
            }
            if case.get("store_full"):
                _write_gz(os.path.join(out_dir, case["name"] + ".tsv.gz"), blob)
                if case["source"]["kind"] == "inline":
                    _write_gz(os.path.join(out_dir, case["name"] + ".in.gz"), data)
            with open(os.path.join(out_dir, case["name"] + ".json"), "w") as f:
                json.dump(fx, f, indent=1, sort_keys=True)
            print(f"{case['name']}: {len(lines)} lines {stats}")
            if case.get("parts"):
                parts = run_ref_parts(case, data, tmp)
                from oracle.oracle import split_records
                pj = {"name": case["name"], "k": case["k"], "m": case["m"], "n": case.get("n", 16),
                      "input_sha256": fx["input_sha256"], "partitions": []}
                for blob_p in parts:
                    recs = sorted(f"{ln:04x}{mp:04x}{pk.hex()}" for ln, mp, pk in
                                  split_records(blob_p, case["k"], case["m"]))
                    h = hashlib.sha256("\n".join(recs).encode()).hexdigest()
                    pj["partitions"].append({"records": len(recs), "bytes": len(blob_p), "sha256": h})
                with open(os.path.join(out_dir, case["name"] + ".parts.json"), "w") as f:
                    json.dump(pj, f, indent=1, sort_keys=True)
                print(f"  partitions: {sum(p['records'] for p in pj['partitions'])} records")


if __name__ == "__main__":
    main()
