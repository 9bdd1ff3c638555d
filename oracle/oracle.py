"""ctypes front end of the CPU oracle (oracle/tuna_oracle.c).

Test infrastructure, not the product: tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it to verify and to time. It restates the reference
tuna counting path (see tuna_oracle.h for the file:line map) and is pinned
against the reference's own outputs in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, List, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libtuna_oracle.so")
SRC = os.path.join(HERE, "tuna_oracle.c")
DIGEST_H = os.path.join(HERE, "tuna_digest.h")
TSV_DIGEST_SRC = os.path.join(HERE, "tsv_digest.c")
TSV_DIGEST_BIN = os.path.join(BUILD, "tsv_digest")

_lib = None


def _stale(target: str, *srcs: str) -> bool:
    return not os.path.exists(target) or any(os.path.getmtime(target) < os.path.getmtime(s) for s in srcs)


def build(force: bool = False) -> str:
    """Compile the oracle shared library and the TSV digester (portable C11,
    no ISA flags)."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = os.path.join(HERE, "tuna_oracle.h")
    if force or _stale(LIB_PATH, SRC, hdr, DIGEST_H):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-shared", "-fPIC", "-pthread",
                               SRC, "-o", tmp])
        os.replace(tmp, LIB_PATH)
    if force or _stale(TSV_DIGEST_BIN, TSV_DIGEST_SRC, DIGEST_H):
        tmp = TSV_DIGEST_BIN + ".tmp"
        subprocess.check_call(["gcc", "-O3", "-std=c11", TSV_DIGEST_SRC, "-o", tmp])
        os.replace(tmp, TSV_DIGEST_BIN)
    return LIB_PATH


class _Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in
                ("n_runs", "n_kmers", "n_superkmers", "n_distinct", "n_out", "record_bytes")]


class _Digest(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("pairs", "count_sum", "h1", "h2")]


def digest_dict(d) -> Dict[str, object]:
    """The digest as stored in the golden fixtures (hashes as 16 hex digits)."""
    return {"pairs": int(d.pairs), "count_sum": int(d.count_sum),
            "h1": f"{int(d.h1):016x}", "h2": f"{int(d.h2):016x}"}


_RUN_CB = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t, ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64, vp, i32 = ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int
        L.tor_parse_fastx.argtypes = [vp, ctypes.c_size_t, _RUN_CB, vp]
        L.tor_parse_fastx.restype = i32
        L.tor_nthash_canonical.argtypes = [vp, i32]
        L.tor_nthash_canonical.restype = u64
        for fn in (L.tor_count_stream, L.tor_count_fastx, L.tor_count_stream_unsorted):
            fn.argtypes = [vp, ctypes.c_size_t, i32, i32, u64, u64, u64, i32, ctypes.POINTER(_Stats)]
            fn.restype = vp
        L.tor_result_words.argtypes = [vp]
        L.tor_result_words.restype = i32
        L.tor_result_size.argtypes = [vp]
        L.tor_result_size.restype = u64
        L.tor_result_keys.argtypes = [vp]
        L.tor_result_keys.restype = ctypes.POINTER(ctypes.c_uint64)
        L.tor_result_counts.argtypes = [vp]
        L.tor_result_counts.restype = ctypes.POINTER(ctypes.c_uint32)
        L.tor_result_free.argtypes = [vp]
        for fn in (L.tor_digest_stream, L.tor_digest_fastx):
            fn.argtypes = [vp, ctypes.c_size_t, i32, i32, u64, u64, u64, i32, ctypes.POINTER(_Stats),
                           ctypes.POINTER(_Digest)]
            fn.restype = i32
        L.tor_result_digest.argtypes = [vp, ctypes.POINTER(_Digest)]
        L.tor_result_digest.restype = None
        L.tor_digest_pairs.argtypes = [vp, i32, i32, vp, u64, ctypes.POINTER(_Digest)]
        L.tor_digest_pairs.restype = None
        L.tor_partition_stream.argtypes = [vp, ctypes.c_size_t, i32, i32, u64, i32]
        L.tor_partition_stream.restype = vp
        L.tor_parts_data.argtypes = [vp]
        L.tor_parts_data.restype = ctypes.POINTER(ctypes.c_uint8)
        L.tor_parts_offsets.argtypes = [vp]
        L.tor_parts_offsets.restype = ctypes.POINTER(ctypes.c_uint64)
        L.tor_parts_free.argtypes = [vp]
        L.tor_write_tsv.argtypes = [vp, i32, ctypes.c_char_p]
        L.tor_write_tsv.restype = i32
        L.tor_write_kff.argtypes = [vp, i32, ctypes.c_char_p]
        L.tor_write_kff.restype = i32
        _lib = L
    return _lib


def _as_u8(data) -> np.ndarray:
    if isinstance(data, (bytes, bytearray, memoryview)):
        return np.frombuffer(bytes(data), dtype=np.uint8)
    a = np.ascontiguousarray(data, dtype=np.uint8)
    return a


def parse_fastx(data) -> List[bytes]:
    """ACGT runs of a FASTA/FASTQ buffer, in order (helicase semantics)."""
    buf = _as_u8(data)
    out: List[bytes] = []

    def cb(p, n, _u):
        out.append(ctypes.string_at(p, n))

    fn = _RUN_CB(cb)
    rc = lib().tor_parse_fastx(buf.ctypes.data if buf.size else None, buf.size, fn, None)
    if rc != 0:
        raise RuntimeError("Empty file")
    return out


def nthash(mmer: bytes) -> int:
    b = _as_u8(mmer)
    return int(lib().tor_nthash_canonical(b.ctypes.data, len(b)))


class Result:
    """Sorted (canonical k-mer, count) pairs. keys: (n, words) uint64, word 0
    holds the last 32 bases; counts: (n,) uint32."""

    def __init__(self, keys: np.ndarray, counts: np.ndarray, stats: Dict[str, int], k: int):
        self.keys, self.counts, self.stats, self.k = keys, counts, stats, k

    def __len__(self) -> int:
        return int(self.counts.shape[0])

    def tsv_lines(self) -> List[str]:
        return [f"{label(self.keys[i], self.k)}\t{int(self.counts[i])}" for i in range(len(self))]


def label(words, k: int) -> str:
    m = "ACGT"
    out = []
    for i in range(k):
        b = k - 1 - i
        out.append(m[(int(words[b >> 5]) >> (2 * (b & 31))) & 3])
    return "".join(out)


def _take(res_ptr, k: int, st: _Stats) -> Result:
    L = lib()
    if not res_ptr:
        raise ValueError("oracle rejected the parameters")
    try:
        nw = L.tor_result_words(res_ptr)
        n = L.tor_result_size(res_ptr)
        keys = np.ctypeslib.as_array(L.tor_result_keys(res_ptr), shape=(max(n, 1) * nw,))[: n * nw]
        keys = keys.reshape(n, nw).copy()
        counts = np.ctypeslib.as_array(L.tor_result_counts(res_ptr), shape=(max(n, 1),))[:n].copy()
    finally:
        L.tor_result_free(res_ptr)
    stats = {f: int(getattr(st, f)) for f, _ in _Stats._fields_}
    return Result(keys, counts, stats, k)


def count_stream(seq, k: int, m: int, n_parts: int = 16, ci: int = 1,
                 cx: int = (1 << 64) - 1, threads: int = 1) -> Result:
    """Count over a sequence stream (any non-ACGT byte separates runs)."""
    buf = _as_u8(seq)
    st = _Stats()
    p = lib().tor_count_stream(buf.ctypes.data if buf.size else None, buf.size, k, m,
                               n_parts, ci, cx, threads, ctypes.byref(st))
    return _take(p, k, st)


def count_stream_unsorted(seq, k: int, m: int, n_parts: int = 16, ci: int = 1,
                          cx: int = (1 << 64) - 1, threads: int = 1) -> Result:
    """count_stream without the final sort (what the CPU baseline times)."""
    buf = _as_u8(seq)
    st = _Stats()
    p = lib().tor_count_stream_unsorted(buf.ctypes.data if buf.size else None, buf.size, k, m,
                                        n_parts, ci, cx, threads, ctypes.byref(st))
    return _take(p, k, st)


def count_fastx(data, k: int, m: int, n_parts: int = 16, ci: int = 1,
                cx: int = (1 << 64) - 1, threads: int = 1) -> Result:
    buf = _as_u8(data)
    if buf.size == 0:
        raise RuntimeError("Empty file")
    st = _Stats()
    p = lib().tor_count_fastx(buf.ctypes.data, buf.size, k, m, n_parts, ci, cx, threads,
                              ctypes.byref(st))
    return _take(p, k, st)


def digest_stream(seq, k: int, m: int, n_parts: int = 16, ci: int = 1,
                  cx: int = (1 << 64) - 1, threads: int = 1, fastx: bool = False):
    """Count a sequence stream (or FASTA/FASTQ bytes with fastx=True) and return
    (digest dict, stats dict) without keeping the pairs: memory for Phase 1's
    records and one partition table per thread, so it scales to the
    full-size workloads."""
    buf = _as_u8(seq)
    if fastx and buf.size == 0:
        raise RuntimeError("Empty file")
    st = _Stats()
    d = _Digest()
    fn = lib().tor_digest_fastx if fastx else lib().tor_digest_stream
    rc = fn(buf.ctypes.data if buf.size else None, buf.size, k, m, n_parts, ci, cx, threads,
            ctypes.byref(st), ctypes.byref(d))
    if rc != 0:
        raise ValueError("oracle rejected the parameters")
    return digest_dict(d), {f: int(getattr(st, f)) for f, _ in _Stats._fields_}


def digest_pairs(keys: np.ndarray, counts: np.ndarray, k: int, threads: int = 1) -> Dict[str, object]:
    """Digest of (keys, counts) arrays held in host memory (keys: (n, words)
    uint64 in the Kmer<k> layout; only the first ceil(k/32) words count),
    computed on `threads` host threads (slices summed mod 2^64)."""
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    n = int(counts.shape[0])
    stride = int(keys.shape[1]) if keys.ndim == 2 else 1
    nw = (k + 31) // 32
    if stride < nw or keys.size < n * stride:
        raise ValueError("keys have fewer words than k needs")
    L = lib()
    nt = max(1, min(int(threads), n >> 20)) if n else 1
    parts = [_Digest() for _ in range(nt)]

    def one(t):
        a, b = n * t // nt, n * (t + 1) // nt
        if b > a:
            L.tor_digest_pairs(keys.ctypes.data + a * stride * 8, stride, nw, counts.ctypes.data + a * 4, b - a,
                               ctypes.byref(parts[t]))

    if nt == 1:
        one(0)
    else:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(nt) as ex:
            list(ex.map(one, range(nt)))
    tot = _Digest()
    mask = (1 << 64) - 1
    for f in ("pairs", "count_sum", "h1", "h2"):
        setattr(tot, f, sum(int(getattr(p, f)) for p in parts) & mask)
    return digest_dict(tot)


def tsv_digest_file(path: str) -> Dict[str, object]:
    """Digest of a TSV file by the C digester (the program the goldens use)."""
    build()
    with open(path, "rb") as f:
        r = subprocess.run([TSV_DIGEST_BIN], stdin=f, capture_output=True, check=True)
    import json
    d = json.loads(r.stdout)
    d.pop("k", None)
    return d


def write_kff_stream(seq, k: int, m: int, path: str, n_parts: int = 16, ci: int = 1,
                     cx: int = (1 << 64) - 1, threads: int = 1) -> int:
    """Count a sequence stream and write the pairs as a KFF file, as the
    reference's kff_output.hpp lays it out; returns the number of pairs."""
    buf = _as_u8(seq)
    st = _Stats()
    L = lib()
    p = L.tor_count_stream(buf.ctypes.data if buf.size else None, buf.size, k, m, n_parts, ci, cx, threads,
                           ctypes.byref(st))
    if not p:
        raise ValueError("oracle rejected the parameters")
    try:
        n = int(L.tor_result_size(p))
        if L.tor_write_kff(p, k, os.fsencode(path)) != 0:
            raise OSError(f"cannot write {path}")
    finally:
        L.tor_result_free(p)
    return n


def partition_stream(seq, k: int, m: int, n_parts: int, threads: int = 1) -> List[bytes]:
    """Phase 1 only: the concatenated records of each partition, in the
    reference's superkmer file layout."""
    buf = _as_u8(seq)
    L = lib()
    p = L.tor_partition_stream(buf.ctypes.data if buf.size else None, buf.size, k, m, n_parts, threads)
    if not p:
        raise ValueError("oracle rejected the parameters")
    try:
        offs = np.ctypeslib.as_array(L.tor_parts_offsets(p), shape=(n_parts + 1,)).copy()
        total = int(offs[-1])
        data = ctypes.string_at(L.tor_parts_data(p), total) if total else b""
    finally:
        L.tor_parts_free(p)
    return [data[int(offs[i]): int(offs[i + 1])] for i in range(n_parts)]


def split_records(blob: bytes, k: int, m: int) -> List[Tuple[int, int, bytes]]:
    """Split a partition's bytes into (len, min_pos, packed) records."""
    hb = 1 if 2 * k - m <= 255 else 2
    out = []
    o = 0
    n = len(blob)
    while o + 2 * hb <= n:
        ln = int.from_bytes(blob[o:o + hb], "little")
        mp = int.from_bytes(blob[o + hb:o + 2 * hb], "little")
        if ln == 0:
            break
        o += 2 * hb
        nb = (ln + 3) // 4
        out.append((ln, mp, bytes(blob[o:o + nb])))
        o += nb
    return out


def write_tsv(res: Result, path: str) -> None:
    """Write via the oracle's writer (k-mer labels upper-case, '\\t', count)."""
    with open(path, "w") as f:
        for line in res.tsv_lines():
            f.write(line + "\n")


def fastx_to_stream(data) -> bytes:
    """Parse FASTA/FASTQ and join the ACGT runs with LF separators (the
    sequence-stream input convention)."""
    return b"".join(r + b"\n" for r in parse_fastx(data))


def tsv_blob(res: Result) -> bytes:
    """Sorted TSV bytes, as `sort` would order the reference's output lines."""
    return "".join(l + "\n" for l in sorted(res.tsv_lines())).encode()
