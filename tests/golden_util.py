"""Helpers shared by the parity tests: load golden fixtures and compare."""
import gzip
import hashlib
import json
import os
from typing import List

from tests.golden import cases as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture(name: str) -> dict:
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def parts_fixture(name: str):
    p = os.path.join(GOLDEN, name + ".parts.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def full_tsv(name: str):
    p = os.path.join(GOLDEN, name + ".tsv.gz")
    if not os.path.exists(p):
        return None
    with gzip.open(p, "rb") as f:
        return f.read()


def case(name: str) -> dict:
    for c in C.CASES + C.SCALE_CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


def case_input(name: str) -> bytes:
    c = case(name)
    data = C.load_input(c)
    fx = fixture(name)
    assert hashlib.sha256(data).hexdigest() == fx["input_sha256"], \
        f"{name}: regenerated input differs from the one the reference ran on"
    return data


def sha(blob: bytes) -> str:
    return hashlib.sha256(blob).hexdigest()


def record_multiset_sha(records) -> str:
    recs = sorted(f"{ln:04x}{mp:04x}{pk.hex()}" for ln, mp, pk in records)
    return hashlib.sha256("\n".join(recs).encode()).hexdigest()


CASE_NAMES: List[str] = [c["name"] for c in C.CASES]
