"""Serving: a continuous-batching request loop over jobs of several samples
(tg_job_next_sample and the job API of include/tuna_gpu.h).

A request is one count job: a sequence stream (non-ACGT bytes separate runs,
as tg_job_feed_seq takes it) or the bytes of a FASTA/FASTQ file (lexed on the
device, tg_job_feed_fastx), and its k, m, ci, cx. Requests are queued as
they arrive. Each of `workers` worker threads owns a device context (its own
CUDA stream and device buffers); whenever a worker is free it takes every
waiting request of the same kind with the same (k, m, ci, cx) as the oldest
one, up to a budget of bases, and counts them as the samples of one job.
Admission is by free device memory at the moment a batch is taken: the
budget is the device's free memory now, plus what this worker's context
already holds, shared among the workers (DEVICE_BYTES_PER_BASE per base).
Requests that arrive while a batch is on the device join a later batch as soon
as a worker frees up; with two workers two batches are in flight, so one
batch's host copies and host work overlap the other's kernels. A job keeps its
samples apart, so every request's result is its result alone.

Results land in page-locked host memory (tg_host_alloc) that each worker keeps
and reuses: a slab holds one batch's pairs (sized by their number, known once
the job has run), the answers of the batch are numpy views of it, and the slab
returns to its worker when the last array viewing it is gone (pinning fresh
memory per batch cost tens of milliseconds to a second for large batches).

The reference has no serving mode (it counts one input set per process run);
this is the request loop around the same counting path.
"""
import ctypes
import threading
import time
import weakref
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


class _Slab:
    """Page-locked host memory of one worker (tg_host_alloc)."""

    def __init__(self, T, nbytes: int):
        self.hb = T.HostBuffer(nbytes)
        self.nbytes = nbytes


class _Pool:
    """A worker's slabs: grow-only, each reused once every view of it is gone."""

    def __init__(self, T):
        self._T = T
        self._free: List[_Slab] = []
        self._mu = threading.Lock()
        self.allocated = 0

    def get(self, nbytes: int) -> "_Lease":
        with self._mu:
            fit = [s for s in self._free if s.nbytes >= nbytes]
            if fit:
                slab = min(fit, key=lambda s: s.nbytes)
                self._free.remove(slab)
            else:
                slab = None
        if slab is None:
            # grow-only: round up so that similar batches reuse the slab
            size = 1 << max(20, (max(1, nbytes) - 1).bit_length())
            slab = _Slab(self._T, size)
            self.allocated += 1
        return _Lease(self, slab)

    def give_back(self, slab: _Slab) -> None:
        with self._mu:
            self._free.append(slab)

    def close(self) -> None:
        with self._mu:
            for s in self._free:
                s.hb.close()
            self._free.clear()


class _Lease:
    """One batch's use of a slab; the slab goes back to the pool when the lease
    (held by every array viewing it) is collected."""

    def __init__(self, pool: _Pool, slab: _Slab):
        self.slab = slab
        weakref.finalize(self, pool.give_back, slab)

    def view(self, offset: int, n: int, dtype) -> np.ndarray:
        dt = np.dtype(dtype)
        if offset + n * dt.itemsize > self.slab.nbytes:
            raise ValueError("view past the slab")
        return np.asarray(_View(self, self.slab.hb.ptr + offset, n, dt))


class _View:
    """numpy array interface over slab memory; keeps the lease alive."""

    def __init__(self, lease: _Lease, ptr: int, n: int, dt: np.dtype):
        self._lease = lease
        self.__array_interface__ = {"data": (ptr, False), "shape": (n,), "typestr": dt.str,
                                    "version": 3}


class Server:
    """max_batch_bases: a fixed budget of bases per batch instead of admission
    by free device memory. paused: workers take nothing until resume() (a
    caller can queue requests first, e.g. to measure merging). slab_bytes:
    page-locked result memory each worker pins when it starts (more is pinned,
    and kept, when a batch needs it)."""

    def __init__(self, device: int = 0, workers: int = 2, max_batch_bases: Optional[int] = None,
                 host_threads: int = 0, paused: bool = False, slab_bytes: int = 1 << 30):
        if workers < 1:
            raise ValueError("a server needs at least one worker")
        import tuna_gb300 as T
        self._T = T
        self._L = T.library()
        self.device = device
        self.workers = workers
        self.slab_bytes = int(slab_bytes)  # page-locked result memory each worker pins at start
        self.max_batch_bases = None if max_batch_bases is None else int(max_batch_bases)
        self._q: Deque[_Req] = deque()
        self._cv = threading.Condition()
        self._stop = False
        self._paused = bool(paused)
        self._alive = workers       # workers that hold a device context
        self._error: Optional[BaseException] = None  # why no worker is left
        self.batches = 0
        self.batch_sizes: List[int] = []   # requests per batch, in the order batches were taken
        self.budgets: List[int] = []       # admission budget (bases) when each batch was taken
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

    def resume(self) -> None:
        """Let the workers take requests (a server made with paused=True)."""
        with self._cv:
            self._paused = False
            self._cv.notify_all()

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._paused = False
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ worker
    def _budget(self, held: int) -> int:
        """Bases one batch may take now: free device memory plus what this
        worker's context already holds (its grow-only buffers are reused),
        shared among the workers."""
        if self.max_batch_bases is not None:
            return self.max_batch_bases
        free = _free_device_bytes(self.device) + held
        return max(1 << 20, int(free * 0.8 / self.workers / DEVICE_BYTES_PER_BASE))

    def _work(self, device: int, host_threads: int) -> None:
        T, L = self._T, self._L
        try:
            ctx = T.Context(device, host_threads, autotune=True)
        except Exception as e:  # noqa: BLE001 - the last worker lost fails every waiting request
            self._worker_lost(e)
            return
        pool = _Pool(T)
        if self.slab_bytes:
            pool.give_back(_Slab(T, self.slab_bytes))  # pinned once, at start
        held = 0  # device bytes this worker's context holds (its largest batch so far)
        try:
            while True:
                with self._cv:
                    while (not self._q or self._paused) and not self._stop:
                        self._cv.wait()
                    if not self._q:
                        return
                    budget = self._budget(held)
                    batch, self._q = take_batch(self._q, budget)
                    self.batches += 1
                    self.batch_sizes.append(len(batch))
                    self.budgets.append(budget)
                held = max(held, DEVICE_BYTES_PER_BASE * sum(int(r.seq.size) for r in batch))
                try:
                    self._run(ctx, pool, batch)
                except Exception as e:  # noqa: BLE001 - every waiting future learns of it
                    for r in batch:
                        if not r.future.done():
                            r.future.set_exception(e)
        finally:
            pool.close()
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

    def _run(self, ctx, pool: "_Pool", batch: List[_Req]) -> None:
        """One batch as one job of several samples (the job API): the pairs stay
        on the device until the job has run, then go to a slab sized by their
        number (at most the pairs bound of tg_count_batch's cap, bases, is
        usually several times too large), copied by the library's host-link
        copy into the page-locked slab."""
        T, L = self._T, self._L
        k, m, ci, cx, fastx = batch[0].key
        W = 1 if k <= 31 else 2
        n = len(batch)
        o = T._JobOpts(k, m, 16, ci, cx, 0, 0)
        j = ctypes.c_void_p()
        ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
        try:
            feed = L.tg_job_feed_fastx if fastx else L.tg_job_feed_seq
            for i, r in enumerate(batch):
                if i:
                    ctx.check(L.tg_job_next_sample(j))
                if r.seq.size:
                    ctx.check(feed(j, ctypes.c_void_p(r.seq.ctypes.data), int(r.seq.size)))
            ctx.check(L.tg_job_run(j))
            n_out = int(L.tg_job_result_size(j))
            lease = pool.get(max(1, n_out) * (8 * W + 4))
            keys = lease.view(0, n_out * W, np.uint64)
            cnt = lease.view(n_out * W * 8, n_out, np.uint32)
            if n_out:
                ctx.check(L.tg_job_result_copy(j, ctypes.c_void_p(keys.ctypes.data), ctypes.c_void_p(cnt.ctypes.data),
                                               0, n_out))
            off = np.zeros(n + 1, dtype=np.uint64)
            ctx.check(L.tg_job_sample_offsets(j, ctypes.c_void_p(off.ctypes.data)))
        finally:
            L.tg_job_end(j)
        done = time.perf_counter()
        kk = keys.reshape(-1, W)
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
