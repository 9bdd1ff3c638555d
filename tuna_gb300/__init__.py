"""tuna_gb300 — GB300-native k-mer counting (tuna's two-phase path).

Python front end over the C ABI of libtuna_gpu.so (include/tuna_gpu.h). It
mirrors the reference library API of include/tuna/tuna.hpp for Python callers:

    count_to_raw(files, k, m, opts)   -> (keys, counts)      tuna::count_to_raw
    count_to(files, k, m, opts)       -> {kmer: count}       tuna::count_to
    count(files, cb, k, m, opts)      cb(kmer, count)        tuna::count
    Options(threads, min_count, max_count, partitions, ...)  tuna::Options

and exposes the lower-level job interface (sequence streams in host or device
memory, raw results, partition export, stats) used by the tests and bench.py.
There is no CPU fallback: without the compiled library or a CUDA device every
call raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import build as _build

__all__ = ["Options", "Context", "GpuError", "count_stream", "count_fastx", "count_to_raw", "count_to",
           "count", "library", "label_array", "tsv_blob"]

_U64_MAX = (1 << 64) - 1

ERRORS = {0: "ok", 1: "bad argument", 2: "CUDA error", 3: "out of memory", 4: "bad state", 5: "I/O error",
          6: "parse error", 7: "table overflow", 8: "device wait gave up", 9: "unsupported"}


class GpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _CtxOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_uint64),
                ("host_threads", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class _JobOpts(ctypes.Structure):
    _fields_ = [("k", ctypes.c_uint16), ("m", ctypes.c_uint16), ("n_parts", ctypes.c_uint32),
                ("ci", ctypes.c_uint64), ("cx", ctypes.c_uint64), ("gpu_parts", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class _Stats(ctypes.Structure):
    _fields_ = [("input_bytes", ctypes.c_uint64), ("bases", ctypes.c_uint64), ("runs", ctypes.c_uint64),
                ("kmers", ctypes.c_uint64), ("superkmers", ctypes.c_uint64), ("distinct", ctypes.c_uint64),
                ("out", ctypes.c_uint64), ("gpu_parts", ctypes.c_uint32), ("heavy_groups", ctypes.c_uint32),
                ("fallback_groups", ctypes.c_uint64), ("h2d_ms", ctypes.c_double), ("pack_ms", ctypes.c_double),
                ("phase1_ms", ctypes.c_double), ("phase2_ms", ctypes.c_double), ("d2h_ms", ctypes.c_double),
                ("phase1_cut_ms", ctypes.c_double), ("phase1_scatter_ms", ctypes.c_double),
                ("record_bytes", ctypes.c_uint64), ("gpu_launches", ctypes.c_uint64),
                ("phase2_count_ms", ctypes.c_double), ("phase2_keys_ms", ctypes.c_double),
                ("groups", ctypes.c_uint64), ("lex_ms", ctypes.c_double), ("fastx_bytes", ctypes.c_uint64),
                ("host_parsed_bytes", ctypes.c_uint64), ("phase2_passes", ctypes.c_uint64),
                ("group_load_pct", ctypes.c_uint32), ("autotune_trials", ctypes.c_uint32)]

    def as_dict(self) -> Dict[str, float]:
        return {f: getattr(self, f) for f, _ in self._fields_}


class _Digest(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_uint64), ("count_sum", ctypes.c_uint64), ("h1", ctypes.c_uint64),
                ("h2", ctypes.c_uint64)]

    def as_dict(self) -> Dict[str, object]:
        """As stored in the golden fixtures: hashes as 16 hex digits."""
        return {"pairs": int(self.pairs), "count_sum": int(self.count_sum), "h1": f"{int(self.h1):016x}",
                "h2": f"{int(self.h2):016x}"}


_PART_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t,
                              ctypes.c_void_p)
_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_void_p)

_lib = None

# Every symbol of include/tuna_gpu.h; tests check the library exports them all.
ABI_SYMBOLS = ["tg_ctx_create", "tg_ctx_destroy", "tg_last_error", "tg_ctx_stream", "tg_version", "tg_device_count",
               "tg_job_begin", "tg_job_feed_seq", "tg_job_feed_seq_device", "tg_job_feed_fastx",
               "tg_job_feed_file", "tg_job_run", "tg_job_stats", "tg_job_result_size", "tg_job_key_words",
               "tg_job_result_copy", "tg_job_drain", "tg_job_write", "tg_job_export_partitions", "tg_job_end",
               "tg_count_seq", "tg_count_seq_device_noalloc", "tg_job_next_sample", "tg_job_sample_count",
               "tg_job_sample_offsets", "tg_count_batch", "tg_job_feed_fastx_device", "tg_count_fastx",
               "tg_fastx_to_stream", "tg_read_input", "tg_count_batch_fastx", "tg_job_set_shard",
               "tg_job_result_digest", "tg_host_alloc", "tg_host_free", "tg_job_set_spill"]


def library(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libtuna_gpu.so (building it in-tree if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.GPU_LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise GpuError(9, f"{path} is missing; run __graft_entry__.build()")
        path = _build.gpu_lib()
    L = ctypes.CDLL(path)
    vp, u64, u32, i32, sz = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_size_t
    L.tg_ctx_create.argtypes = [ctypes.POINTER(_CtxOpts), ctypes.POINTER(vp)]
    L.tg_ctx_destroy.argtypes = [vp]
    L.tg_last_error.argtypes = [vp]
    L.tg_last_error.restype = ctypes.c_char_p
    L.tg_ctx_stream.argtypes = [vp]
    L.tg_ctx_stream.restype = vp
    L.tg_version.restype = ctypes.c_char_p
    L.tg_device_count.restype = i32
    L.tg_job_begin.argtypes = [vp, ctypes.POINTER(_JobOpts), ctypes.POINTER(vp)]
    L.tg_job_feed_seq.argtypes = [vp, vp, sz]
    L.tg_job_feed_seq_device.argtypes = [vp, vp, sz]
    L.tg_job_feed_fastx.argtypes = [vp, vp, sz]
    L.tg_job_feed_file.argtypes = [vp, ctypes.c_char_p]
    L.tg_job_feed_fastx_device.argtypes = [vp, vp, sz]
    L.tg_count_fastx.argtypes = [vp, ctypes.POINTER(_JobOpts), vp, sz, vp, vp, u64, ctypes.POINTER(u64),
                                 ctypes.POINTER(_Stats)]
    L.tg_fastx_to_stream.argtypes = [vp, vp, sz, vp, sz, ctypes.POINTER(sz)]
    L.tg_read_input.argtypes = [ctypes.c_char_p, u32, vp, sz, ctypes.POINTER(sz), ctypes.c_char_p, sz]
    L.tg_count_batch_fastx.argtypes = [vp, ctypes.POINTER(_JobOpts), u32, ctypes.POINTER(vp), ctypes.POINTER(sz), vp,
                                       vp, vp, u64, ctypes.POINTER(u64), ctypes.POINTER(_Stats)]
    L.tg_job_run.argtypes = [vp]
    L.tg_job_stats.argtypes = [vp, ctypes.POINTER(_Stats)]
    L.tg_job_result_size.argtypes = [vp]
    L.tg_job_result_size.restype = u64
    L.tg_job_key_words.argtypes = [vp]
    L.tg_job_key_words.restype = i32
    L.tg_job_result_copy.argtypes = [vp, vp, vp, u64, u64]
    L.tg_job_drain.argtypes = [vp, i32, _SINK, vp]
    L.tg_job_write.argtypes = [vp, i32, ctypes.c_char_p]
    L.tg_job_export_partitions.argtypes = [vp, _PART_SINK, vp]
    L.tg_job_end.argtypes = [vp]
    L.tg_count_seq.argtypes = [vp, ctypes.POINTER(_JobOpts), vp, sz, vp, vp, u64, ctypes.POINTER(u64),
                               ctypes.POINTER(_Stats)]
    L.tg_count_seq_device_noalloc.argtypes = [ctypes.POINTER(_JobOpts), vp, sz, vp, vp, u64,
                                              ctypes.POINTER(u64), vp, ctypes.c_char_p, sz]
    L.tg_count_seq_device_noalloc.restype = i32
    L.tg_job_next_sample.argtypes = [vp]
    L.tg_job_sample_count.argtypes = [vp]
    L.tg_job_sample_count.restype = u32
    L.tg_job_sample_offsets.argtypes = [vp, vp]
    L.tg_job_set_shard.argtypes = [vp, u32, u32]
    L.tg_job_result_digest.argtypes = [vp, u64, u64, ctypes.POINTER(_Digest)]
    L.tg_host_alloc.argtypes = [sz, ctypes.POINTER(vp)]
    L.tg_job_set_spill.argtypes = [vp, u64, ctypes.c_char_p]
    L.tg_host_free.argtypes = [vp]
    L.tg_count_batch.argtypes = [vp, ctypes.POINTER(_JobOpts), u32, ctypes.POINTER(vp), ctypes.POINTER(sz), vp, vp,
                                 vp, u64, ctypes.POINTER(u64), ctypes.POINTER(_Stats)]
    for fn in ("tg_ctx_create", "tg_ctx_destroy", "tg_job_begin", "tg_job_feed_seq", "tg_job_feed_seq_device",
               "tg_job_feed_fastx", "tg_job_feed_file", "tg_job_run", "tg_job_stats", "tg_job_result_copy",
               "tg_job_drain", "tg_job_write", "tg_job_export_partitions", "tg_job_end", "tg_count_seq",
               "tg_job_next_sample", "tg_job_sample_offsets", "tg_count_batch", "tg_job_feed_fastx_device",
               "tg_count_fastx", "tg_fastx_to_stream", "tg_read_input", "tg_count_batch_fastx",
               "tg_job_set_shard", "tg_job_result_digest", "tg_host_alloc", "tg_host_free", "tg_job_set_spill"):
        getattr(L, fn).restype = i32
    _lib = L
    return L


@dataclass
class Options:
    """tuna::Options (include/tuna/tuna.hpp:59-66)."""
    threads: int = 1
    min_count: int = 1
    max_count: int = (1 << 32) - 1
    partitions: int = 0
    ram_gb: int = 0
    work_dir: str = ""


@dataclass
class Result:
    keys: np.ndarray          # (n, words) uint64, Kmer<k> word layout
    counts: np.ndarray        # (n,) uint32
    stats: Dict[str, float] = field(default_factory=dict)
    k: int = 0
    samples: Optional[np.ndarray] = None  # (n,) uint32 sample of each pair (jobs of several samples)
    formatted: Optional[bytes] = None     # tg_job_drain output, when asked for
    digest: Optional[Dict[str, object]] = None  # tg_job_result_digest of all pairs, when asked for
    sample_digests: Optional[List[Dict[str, object]]] = None  # per sample (jobs of several samples)

    def __len__(self) -> int:
        return int(self.counts.shape[0])

    def sorted(self) -> "Result":
        order = np.lexsort(tuple(self.keys[:, i] for i in range(self.keys.shape[1])))
        return Result(self.keys[order], self.counts[order], self.stats, self.k,
                      None if self.samples is None else self.samples[order])

    def sample(self, i: int) -> "Result":
        """The pairs of sample i (all pairs for a job of one sample)."""
        if self.samples is None:
            return self
        sel = self.samples == i
        return Result(self.keys[sel], self.counts[sel], self.stats, self.k)


def label_array(keys: np.ndarray, k: int) -> np.ndarray:
    """(n, k) uint8 ASCII labels of (n, words) keys (vectorised get_label)."""
    n = keys.shape[0]
    out = np.empty((n, k), dtype=np.uint8)
    lut = np.frombuffer(b"ACGT", dtype=np.uint8)
    for i in range(k):
        b = k - 1 - i
        out[:, i] = lut[((keys[:, b >> 5] >> np.uint64(2 * (b & 31))) & np.uint64(3)).astype(np.intp)]
    return out


def tsv_blob(keys: np.ndarray, counts: np.ndarray, k: int) -> bytes:
    """Sorted TSV bytes ("<kmer>\\t<count>\\n"), lines in byte order as `sort`."""
    if len(counts) == 0:
        return b""
    lab = label_array(keys, k)
    cs = counts.astype(np.uint64)
    digits = np.char.mod("%d", cs).astype(f"S{10}")
    lines = np.char.add(np.char.add(lab.view(f"S{k}").ravel(), b"\t"), digits)
    lines = np.sort(lines)
    return b"\n".join(lines.tolist()) + b"\n"


class Context:
    """One device context (tg_ctx): a stream and grow-only device buffers that
    consecutive jobs reuse."""

    def __init__(self, device: int = 0, host_threads: int = 0, hbm_budget: int = 0, autotune: bool = False):
        """hbm_budget: device bytes phase 2 may hold at once (0 = free HBM minus
        a reserve); a job whose keys and pairs exceed it runs in passes over
        ranges of bins. autotune: TG_CTX_AUTOTUNE (group size timed on the
        first large job of each key width)."""
        L = library()
        if L.tg_device_count() <= device:
            raise GpuError(2, "no CUDA device available for the GPU k-mer counter")
        self._L = L
        o = _CtxOpts(device, hbm_budget, host_threads, 1 if autotune else 0)
        h = ctypes.c_void_p()
        rc = L.tg_ctx_create(ctypes.byref(o), ctypes.byref(h))
        if rc != 0:
            raise GpuError(rc, "tg_ctx_create failed")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.tg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream_ptr(self) -> int:
        """cudaStream_t of this context (all library work runs on it)."""
        return int(self._L.tg_ctx_stream(self.h) or 0)

    def check(self, rc: int) -> None:
        if rc != 0:
            raise GpuError(rc, self._L.tg_last_error(self.h).decode(errors="replace"))

    # ------------------------------------------------------------------ jobs
    def _opts(self, k, m, n_parts, ci, cx, gpu_parts) -> _JobOpts:
        return _JobOpts(k, m, n_parts, ci, min(cx, _U64_MAX), gpu_parts, 0)

    def lex(self, data) -> bytes:
        """FASTA/FASTQ bytes to the sequence stream, lexed on the device
        (tg_fastx_to_stream)."""
        a = np.ascontiguousarray(np.frombuffer(data, dtype=np.uint8) if isinstance(data, (bytes, bytearray))
                                 else data, dtype=np.uint8)
        out = np.empty(max(1, a.size + 1), dtype=np.uint8)
        n = ctypes.c_size_t()
        self.check(self._L.tg_fastx_to_stream(self.h, a.ctypes.data if a.size else None, a.size, out.ctypes.data,
                                              out.size, ctypes.byref(n)))
        return out[: n.value].tobytes()

    def run(self, k: int, m: int, *, seq=None, dev_seq=None, dev_len: int = 0, fastx=None, files=(),
            dev_fastx=None, samples=None, n_parts: int = 16, ci: int = 1, cx: int = _U64_MAX, gpu_parts: int = 0,
            export: bool = False, want_results: bool = True, drain: Optional[int] = None,
            shard: Optional[tuple] = None, digest: bool = False, spill: Optional[tuple] = None):
        """Run one job. seq: host stream (bytes / uint8 array); dev_seq: device
        pointer (int) of dev_len bytes; fastx: FASTA/FASTQ bytes; dev_fastx: device
        pointer of dev_len FASTA/FASTQ bytes; files: paths;
        samples: host streams counted as separate samples of the job (the
        Result then carries the sample of each pair); drain: a tg_format (0 TSV,
        1 KFF entries, 2 RAW) whose bytes tg_job_drain hands back in
        Result.formatted; shard: (s, n) counts only shard s of n of the bins
        (tg_job_set_shard), whose pairs the n shards' results split between them;
        digest: Result.digest (and per sample, Result.sample_digests) from
        tg_job_result_digest; spill: (chunk_bytes, dir or None) runs the job in
        spill mode (tg_job_set_spill: phase 1 per chunk, records to host memory
        or files under dir, phase 2 in passes). Returns (Result, partitions or
        None)."""
        L = self._L
        o = self._opts(k, m, n_parts, ci, cx, gpu_parts)
        j = ctypes.c_void_p()
        self.check(L.tg_job_begin(self.h, ctypes.byref(o), ctypes.byref(j)))
        try:
            if shard is not None:
                self.check(L.tg_job_set_shard(j, int(shard[0]), int(shard[1])))
            if spill is not None:
                d = spill[1] if len(spill) > 1 else None
                self.check(L.tg_job_set_spill(j, int(spill[0]), os.fsencode(d) if d else None))
            for i, smp in enumerate(samples or ()):
                if i:
                    self.check(L.tg_job_next_sample(j))
                a = np.ascontiguousarray(np.frombuffer(smp, dtype=np.uint8) if isinstance(smp, (bytes, bytearray))
                                         else smp, dtype=np.uint8)
                self.check(L.tg_job_feed_seq(j, a.ctypes.data if a.size else None, a.size))
            if seq is not None:
                a = np.ascontiguousarray(np.frombuffer(seq, dtype=np.uint8) if isinstance(seq, (bytes, bytearray))
                                         else seq, dtype=np.uint8)
                self.check(L.tg_job_feed_seq(j, a.ctypes.data if a.size else None, a.size))
            if dev_seq is not None:
                self.check(L.tg_job_feed_seq_device(j, ctypes.c_void_p(dev_seq), dev_len))
            if dev_fastx is not None:
                self.check(L.tg_job_feed_fastx_device(j, ctypes.c_void_p(dev_fastx), dev_len))
            if fastx is not None:
                a = np.frombuffer(fastx, dtype=np.uint8) if isinstance(fastx, (bytes, bytearray)) else fastx
                a = np.ascontiguousarray(a, dtype=np.uint8)
                self.check(L.tg_job_feed_fastx(j, a.ctypes.data if a.size else None, a.size))
            for f in files:
                self.check(L.tg_job_feed_file(j, os.fsencode(f)))
            self.check(L.tg_job_run(j))
            st = _Stats()
            self.check(L.tg_job_stats(j, ctypes.byref(st)))
            n = int(L.tg_job_result_size(j))
            W = int(L.tg_job_key_words(j))
            keys = np.empty((n, W), dtype=np.uint64)
            counts = np.empty(n, dtype=np.uint32)
            smp = None
            if want_results and n:
                self.check(L.tg_job_result_copy(j, keys.ctypes.data, counts.ctypes.data, 0, n))
            dg, sdg = None, None
            if digest:
                d = _Digest()
                self.check(L.tg_job_result_digest(j, 0, n, ctypes.byref(d)))
                dg = d.as_dict()
            if samples is not None and len(samples) > 1:
                off = np.zeros(len(samples) + 1, dtype=np.uint64)
                self.check(L.tg_job_sample_offsets(j, off.ctypes.data))
                smp = np.repeat(np.arange(len(samples), dtype=np.uint32), np.diff(off).astype(np.int64))
                if digest:
                    sdg = []
                    for i in range(len(samples)):
                        d = _Digest()
                        self.check(L.tg_job_result_digest(j, int(off[i]), int(off[i + 1] - off[i]), ctypes.byref(d)))
                        sdg.append(d.as_dict())
            formatted = None
            if drain is not None:
                chunks = []

                def dsink(data, nbytes, _npairs, _u):
                    chunks.append(ctypes.string_at(data, nbytes))
                    return 0

                dcb = _SINK(dsink)
                self.check(L.tg_job_drain(j, int(drain), dcb, None))
                formatted = b"".join(chunks)
            parts = None
            if export:
                parts = [b""] * n_parts

                def sink(p, data, ln, _u):
                    parts[p] = ctypes.string_at(data, ln) if ln else b""
                    return 0

                cb = _PART_SINK(sink)
                self.check(L.tg_job_export_partitions(j, cb, None))
            return Result(keys, counts, st.as_dict(), k, smp, formatted, dg, sdg), parts
        finally:
            L.tg_job_end(j)

    def write(self, k: int, m: int, path: str, *, fastx=None, files=(), fmt: int = 0, n_parts: int = 16,
              ci: int = 1, cx: int = _U64_MAX) -> Dict[str, float]:
        """Count and write TSV (fmt 0) or KFF (fmt 1) to path."""
        L = self._L
        o = self._opts(k, m, n_parts, ci, cx, 0)
        j = ctypes.c_void_p()
        self.check(L.tg_job_begin(self.h, ctypes.byref(o), ctypes.byref(j)))
        try:
            if fastx is not None:
                a = np.ascontiguousarray(np.frombuffer(fastx, dtype=np.uint8) if isinstance(fastx, bytes) else fastx)
                self.check(L.tg_job_feed_fastx(j, a.ctypes.data if a.size else None, a.size))
            for f in files:
                self.check(L.tg_job_feed_file(j, os.fsencode(f)))
            self.check(L.tg_job_run(j))
            self.check(L.tg_job_write(j, fmt, os.fsencode(path)))
            st = _Stats()
            self.check(L.tg_job_stats(j, ctypes.byref(st)))
            return st.as_dict()
        finally:
            L.tg_job_end(j)


class HostBuffer:
    """Page-locked host memory from tg_host_alloc: .array(dtype, count) views it
    as numpy; close() frees it."""

    def __init__(self, nbytes: int):
        L = library()
        p = ctypes.c_void_p()
        rc = L.tg_host_alloc(max(1, int(nbytes)), ctypes.byref(p))
        if rc != 0:
            raise GpuError(rc, f"tg_host_alloc({nbytes}) failed")
        self.ptr, self.nbytes, self._L = int(p.value), int(nbytes), L

    def array(self, dtype=np.uint8, count: Optional[int] = None) -> np.ndarray:
        dt = np.dtype(dtype)
        n = self.nbytes // dt.itemsize if count is None else int(count)
        if n * dt.itemsize > self.nbytes:
            raise ValueError("view larger than the buffer")
        buf = (ctypes.c_uint8 * (n * dt.itemsize)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dt, count=n)

    def close(self) -> None:
        if self.ptr:
            self._L.tg_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def read_input(path: str, threads: int = 0, cap: Optional[int] = None) -> bytes:
    """The bytes of one input file as the library reads it (tg_read_input):
    plain, or inflated for ".gz" (BGZF on `threads` host threads)."""
    L = library()
    if cap is None:
        cap = max(1 << 20, 64 * os.path.getsize(path)) if os.path.exists(path) else 1 << 20
    n = ctypes.c_size_t()
    err = ctypes.create_string_buffer(512)
    for _ in range(2):  # a short buffer is answered with the size needed: read again once
        out = np.empty(cap, dtype=np.uint8)
        rc = L.tg_read_input(os.fsencode(path), threads, out.ctypes.data, cap, ctypes.byref(n), err, 512)
        if rc == 1 and n.value > cap:
            cap = n.value
            continue
        break
    if rc != 0:
        raise GpuError(rc, err.value.decode(errors="replace"))
    return out[: n.value].tobytes()


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def count_stream(seq, k: int, m: int, **kw) -> Result:
    """Count a host sequence stream (non-ACGT bytes separate runs)."""
    return default_context().run(k, m, seq=seq, **kw)[0]


def count_fastx(data, k: int, m: int, **kw) -> Result:
    return default_context().run(k, m, fastx=data, **kw)[0]


def _cx(opts: Options) -> int:
    return int(opts.max_count)


def count_to_raw(files: Sequence[str], k: int, m: int = 21, opts: Optional[Options] = None):
    """tuna::count_to_raw: (keys, counts) of every canonical k-mer within
    [min_count, max_count]."""
    opts = opts or Options()
    if not files:
        raise ValueError("tuna::count: no input files")
    r, _ = default_context().run(k, m, files=list(files), ci=opts.min_count, cx=_cx(opts),
                                 n_parts=opts.partitions or 16)
    return r.keys, r.counts


def count_to(files: Sequence[str], k: int, m: int = 21, opts: Optional[Options] = None) -> Dict[str, int]:
    """tuna::count_to: {kmer label: count}."""
    keys, counts = count_to_raw(files, k, m, opts)
    lab = label_array(keys, k)
    return {bytes(lab[i]).decode(): int(counts[i]) for i in range(len(counts))}


def count(files: Sequence[str], cb: Callable[[str, int], None], k: int, m: int = 21,
          opts: Optional[Options] = None) -> None:
    """tuna::count with an ASCII callback cb(kmer, count)."""
    for kmer, c in count_to(files, k, m, opts).items():
        cb(kmer, c)
