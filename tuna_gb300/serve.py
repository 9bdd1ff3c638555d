"""Serving: a continuous-batching request loop over the batched entry point
(tg_count_batch, include/tuna_gpu.h).

A request is one count job: a sequence stream (non-ACGT bytes separate runs,
as tg_job_feed_seq takes it) or the bytes of a FASTA/FASTQ file (lexed on the
device, tg_count_batch_fastx), and its k, m, ci, cx. Requests are queued as
they arrive. Each of `workers` worker threads owns a device context (its own
CUDA stream and device buffers); whenever a worker is free it takes every
waiting request of the same kind with the same (k, m, ci, cx) as the oldest
one, up to a budget of
bases sized from the free device memory, and counts them as the samples of one
job. Requests that arrive while a batch is on the device join a later batch
as soon as a worker frees up; with two workers two batches are in flight, so
one batch's host copies and host work overlap the other's kernels. A job keeps
its samples apart, so every request's result is its result alone.

The reference has no serving mode (it counts one input set per process run);
this is the request loop around the same counting path.
"""
import ctypes
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Deque, List, Optional, Tuple

import numpy as np

U64_MAX = (1 << 64) - 1
DEVICE_BYTES_PER_BASE = 32  # device memory one input base may take in a job (keys, pairs, descriptors, stream)


@dataclass
class Answer:
    """Result of one request: its (k-mer, count) pairs (Kmer<k> word layout)."""
    keys: np.ndarray
    counts: np.ndarray
    arrival: float     # time.perf_counter() at submit
    done: float        # when the result was ready
    batch: int         # requests counted in the same job

    @property
    def latency_s(self) -> float:
        return self.done - self.arrival


@dataclass
class _Req:
    seq: np.ndarray
    key: Tuple[int, int, int, int, bool]  # k, m, ci, cx, FASTA/FASTQ bytes
    arrival: float
    future: Future = field(default_factory=Future)


def _pinned(n: int, dtype):
    """Page-locked host array of n items (torch's pinned allocator when present),
    else an ordinary numpy array."""
    try:
        import torch
        tdt = {np.uint64: torch.int64, np.uint32: torch.int32, np.uint8: torch.uint8}[dtype]
        return torch.empty(max(n, 1), dtype=tdt, pin_memory=True).numpy().view(dtype)[:n]
    except Exception:
        return np.empty(max(n, 1), dtype=dtype)[:n]


class Server:
    def __init__(self, device: int = 0, workers: int = 2, max_batch_bases: Optional[int] = None,
                 host_threads: int = 0):
        if workers < 1:
            raise ValueError("a server needs at least one worker")
        import tuna_gb300 as T
        self._T = T
        self._L = T.library()
        if max_batch_bases is None:
            free = _free_device_bytes(device)
            max_batch_bases = max(1 << 20, int(free * 0.8 / max(1, workers) / DEVICE_BYTES_PER_BASE))
        self.max_batch_bases = int(max_batch_bases)
        self._q: Deque[_Req] = deque()
        self._cv = threading.Condition()
        self._stop = False
        self._alive = workers       # workers that hold a device context
        self._error: Optional[BaseException] = None  # why no worker is left
        self.batches = 0
        self._threads = [threading.Thread(target=self._work, args=(device, host_threads), daemon=True)
                         for _ in range(workers)]
        for t in self._threads:
            t.start()

    # ------------------------------------------------------------------ API
    def submit(self, seq: np.ndarray, k: int, m: int, ci: int = 1, cx: int = U64_MAX, fastx: bool = False) -> Future:
        """Queue one count job; the future's result is an Answer. fastx: seq is
        the bytes of a FASTA/FASTQ file (lexed on the device), not a stream."""
        if fastx and np.asarray(seq).size == 0:
            raise ValueError("Empty file")
        r = _Req(np.ascontiguousarray(seq, dtype=np.uint8), (k, m, ci, min(cx, U64_MAX), bool(fastx)),
                 time.perf_counter())
        with self._cv:
            if self._stop:
                raise RuntimeError("server is closed")
            if self._error is not None:
                raise RuntimeError(f"no worker could open a device context: {self._error}")
            self._q.append(r)
            self._cv.notify()
        return r.future

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ worker
    def _take(self) -> List[_Req]:
        batch, self._q = take_batch(self._q, self.max_batch_bases)
        return batch

    def _work(self, device: int, host_threads: int) -> None:
        T, L = self._T, self._L
        try:
            ctx = T.Context(device, host_threads, autotune=True)
        except Exception as e:  # noqa: BLE001 - the last worker lost fails every waiting request
            self._worker_lost(e)
            return
        try:
            while True:
                with self._cv:
                    while not self._q and not self._stop:
                        self._cv.wait()
                    if not self._q:
                        return
                    batch = self._take()
                    self.batches += 1
                try:
                    self._run(ctx, batch)
                except Exception as e:  # noqa: BLE001 - every waiting future learns of it
                    for r in batch:
                        if not r.future.done():
                            r.future.set_exception(e)
        finally:
            ctx.close()

    def _worker_lost(self, e: BaseException) -> None:
        with self._cv:
            self._alive -= 1
            if self._alive > 0:
                return
            self._error = e
            while self._q:
                r = self._q.popleft()
                if not r.future.done():
                    r.future.set_exception(e)
            self._cv.notify_all()

    def _run(self, ctx, batch: List[_Req]) -> None:
        T, L = self._T, self._L
        k, m, ci, cx, fastx = batch[0].key
        W = 1 if k <= 31 else 2
        n = len(batch)
        ptrs = (ctypes.c_void_p * n)(*[r.seq.ctypes.data if r.seq.size else None for r in batch])
        lens = (ctypes.c_size_t * n)(*[int(r.seq.size) for r in batch])
        cap = max(1, sum(int(r.seq.size) for r in batch))  # pairs <= k-mer instances < bases
        keys = _pinned(cap * W, np.uint64)
        cnt = _pinned(cap, np.uint32)
        off = np.zeros(n + 1, dtype=np.uint64)
        o = T._JobOpts(k, m, 16, ci, cx, 0, 0)
        n_out = ctypes.c_uint64()
        st = T._Stats()
        fn = L.tg_count_batch_fastx if fastx else L.tg_count_batch
        rc = fn(ctx.h, ctypes.byref(o), n, ptrs, lens, ctypes.c_void_p(keys.ctypes.data),
                ctypes.c_void_p(cnt.ctypes.data), ctypes.c_void_p(off.ctypes.data), cap,
                ctypes.byref(n_out), ctypes.byref(st))
        ctx.check(rc)
        done = time.perf_counter()
        kk = keys[: int(n_out.value) * W].reshape(-1, W)
        for i, r in enumerate(batch):
            a, b = int(off[i]), int(off[i + 1])
            r.future.set_result(Answer(kk[a:b], cnt[a:b], r.arrival, done, n))


def take_batch(queue, max_bases: int):
    """The next batch and the requests left waiting: the oldest request and every
    waiting one of the same kind and parameters, in arrival order, while the
    batch stays within max_bases bases (the oldest always goes, whatever its
    size); the others keep their order."""
    if not queue:
        return [], deque()
    head = queue[0]
    batch, rest, bases = [], deque(), 0
    for r in queue:
        if r.key == head.key and (not batch or bases + r.seq.size <= max_bases):
            batch.append(r)
            bases += r.seq.size
        else:
            rest.append(r)
    return batch, rest


def _free_device_bytes(device: int) -> int:
    try:
        import torch
        free, _ = torch.cuda.mem_get_info(device)
        return int(free)
    except Exception:
        return 64 << 30
