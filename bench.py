#!/usr/bin/env python3
"""bench.py — k-mer counting throughput of the GB300 path.

Workload (one "step"): count every canonical 31-mer (m = 23, tuna -n 4096) of
a seeded synthetic 3.1 Gbp repetitive assembly — 24 contigs of 50-250 Mbp,
GC 41%, 45% of the sequence from 300 bp / 6 kbp repeat families at 10-20%
divergence, 3% microsatellites — the largest single-GPU workload of the
benchmark set. Inputs (3.1 GB) are larger than L2, so no flush is needed.

  value   Gbases/s with the input already resident in HBM: k_pack -> k_cut_fixed/k_cut_seq
          -> k_scan -> k_plan -> k_keys -> k_count, results left on the device
          (stats also give distinct k-mers/s and k-mer updates/s)
  e2e     the same through the public C ABI from the FASTA file's bytes
          (tg_count_fastx) with pinned host buffers: H2D of the FASTA, lexing
          on the device, both phases, D2H of every counted (k-mer, count) pair;
          e2e_stream: the same from the parsed stream (tg_count_seq)
  roofline  the dominant kernel's algorithmic bytes / its CUDA-event time
  cpu_baseline  the CPU oracle (a port of the reference path) on a bounded
          sample of the same workload, all host cores

--impl reference times the CPU port alone (the reference's own sources and
binaries are not present where the bench runs) and prints the same line with "impl": "reference".
Multi-GPU (--gpus N under torchrun): replicas, each rank counts its own copy.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-mer count Gbases/s at k=31 (batched vs plain, 1 GB300); serve p50/p99 ms"
UNIT = "Gbases/s"
K, M, NPARTS = 31, 23, 4096


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the 3.1 Gbp workload")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-plain section")
    ap.add_argument("--no-serve", action="store_true", help="skip the served section")
    ap.add_argument("--no-output", action="store_true", help="skip the output-formatting section")
    ap.add_argument("--no-large-k", action="store_true", help="skip the k=63 reads section")
    ap.add_argument("--large-k-scale", type=float, default=1.0, help="fraction of the 3 Gbp k=63 read set")
    ap.add_argument("--no-gz", action="store_true", help="skip the gzip-input section")
    ap.add_argument("--no-small", action="store_true", help="skip the small read-set section")
    ap.add_argument("--no-passes", action="store_true", help="skip the memory-budget (passes) section")
    ap.add_argument("--batch-samples", type=int, default=2000)
    ap.add_argument("--batch-scales", default="0.004,0.02,0.05",
                    help="genome sizes of the batched mix: log-uniform 10 kbp - 50 Mbp times each of these")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="length of the arrival trace")
    ap.add_argument("--serve-scale", type=float, default=1.0, help="request sizes: median 20 Mbp times this")
    ap.add_argument("--no-autotune", action="store_true",
                    help="group size fixed at half the table (profiling: no trial launches in the warm-up step)")
    ap.add_argument("--no-parity-cpu", action="store_true",
                    help="skip the oracle port's digest of the full-size results (about 30 s of host work each)")
    ap.add_argument("--cpu-mbp", type=float, default=1200.0,
                    help="CPU baseline sample: the first this many Mbp of the assembly (about 10 s on 16 cores)")
    ap.add_argument("--ref-mbp", type=float, default=400.0,
                    help="reference arm, per step: the first this many Mbp of the assembly (a few seconds)")
    return ap.parse_args()


def golden(name: str):
    """A digest fixture of tests/golden (the reference binary's output over the
    same seeded input, recorded by tests/golden/make_golden.py --scale)."""
    path = os.path.join(ROOT, "tests", "golden", name + ".json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def parity_against(device_digest, data, name: str, cpu_digest=None):
    """Key-level parity of one result: its device digest against the
    reference's digest for the same input bytes (when the input's sha256 equals
    the one the reference ran on) and against the oracle port's digest computed
    here (cpu_digest)."""
    import hashlib
    g = golden(name)
    out = {"device_digest": device_digest, "reference_fixture": name}
    if g is not None and data is not None:
        same_input = hashlib.sha256(memoryview(data)).hexdigest() == g["input_sha256"]
        out["input_matches_reference_run"] = same_input
        if same_input:
            out["reference_digest"] = g["digest"]
            out["device_vs_reference"] = device_digest == g["digest"]
    if cpu_digest is not None:
        out["oracle_digest"] = cpu_digest
        out["device_vs_oracle"] = device_digest == cpu_digest
    checks = [out[k2] for k2 in ("device_vs_reference", "device_vs_oracle") if k2 in out]
    out["ok"] = bool(checks) and all(checks)
    return out


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        with open(self.path) as f:
            out = parse_clock_lines(f)
        os.remove(self.path)
        return out


def parse_clock_lines(lines):
    """Median SM clock, maximum clock and throttle reasons seen in nvidia-smi
    samples (ClockSampler.FIELDS, csv, noheader, nounits)."""
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in lines:
        parts = [p.strip() for p in line.split(",")]
        if len(parts) < 9:
            continue
        try:
            clk = float(parts[1])
            top = float(parts[2])
        except ValueError:
            continue
        sm.append(clk)
        mx = top
        for nm, v in zip(names, parts[5:9]):
            if v.lower() in ("active", "yes", "1"):
                reasons.add(nm)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
            "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ workload
def workload(scale: float, want_fasta: bool = True):
    """Sequence stream of the synthetic assembly (contigs separated by LF), the
    number of sequence bases, the contig lengths and the bytes of its 60-column
    FASTA file. The stream is exactly what the reference's FASTA parser hands
    to Phase 1 for that file."""
    import numpy as np
    from tuna_gb300 import synth
    g, lens = synth.repetitive_genome(scale=scale)
    fa = synth.fasta(g, lens) if want_fasta else None
    ends = np.cumsum(lens.astype(np.int64))
    stream = np.insert(g, ends[:-1], np.uint8(10))
    stream = np.append(stream, np.uint8(10))
    return stream, int(g.size), [int(x) for x in lens], fa


def main_config(bases: int, n_stream: int, world: int) -> dict:
    """The workload as both arms name it (identical in the GB300 and the
    reference lines; arm-specific details go in their own keys)."""
    return {"workload": f"{bases / 1e9:.2f} Gbp repetitive assembly, 24 contigs, k=31 m=23 n=4096",
            "k": K, "m": M, "n_parts": NPARTS, "bases": bases, "stream_bytes": n_stream,
            "l2": "inputs larger than L2 (3.1 GB), no flush", "parallelism": f"replicas x{world}"}


def cpu_sample(stream: np.ndarray, mbp: float, threads: int):
    """The first `mbp` Mbp of the assembly's sequence stream, cut into `threads`
    shards (one separator byte between two): the reference's best CPU mode for
    one large file is the same data pre-split into one plain file per core
    (phase 1 in parallel over files, src/partition_hash.hpp:271-279)."""
    seq = stream[stream != 10]
    total = min(int(mbp * 1e6), int(seq.size))
    shard = max(1, total // threads)
    cuts = np.arange(shard, total, shard)
    s = np.insert(seq[:total], cuts, np.uint8(10))
    return np.append(s, np.uint8(10)), total


def time_cpu(threads: int, sample, steps: int = 1, warmup: int = 0):
    """Median seconds of `steps` runs of the oracle port over the CPU sample
    (after `warmup` untimed runs; at least a short warm-up of the library)."""
    from oracle import oracle as O
    s, bases = sample
    O.count_stream_unsorted(s[: min(s.size, 2_000_000)], K, M, NPARTS, threads=threads)  # load, warm
    for _ in range(warmup):
        O.count_stream_unsorted(s, K, M, n_parts=NPARTS, threads=threads)
    ts = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        r = O.count_stream_unsorted(s, K, M, n_parts=NPARTS, threads=threads)
        ts.append(time.perf_counter() - t0)
    t = statistics.median(ts)
    return {"value": bases / t / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the first {bases / 1e6:.0f} Mbp of the same assembly ({bases / 3.1e9:.3f} of it) cut into "
                      f"{threads} shards, k={K} m={M} n={NPARTS}; phase 1 parallel over shards, phase 2 over "
                      f"partitions (the reference's best mode for one large file)",
            "seconds": t, "distinct": len(r)}


# ------------------------------------------------------------------ batched and served
_HOST_BUFS = []


def host_array(n: int, dtype=np.uint8, like=None) -> np.ndarray:
    """n elements of page-locked host memory from the library's allocator
    (tg_host_alloc); with `like`, a copy of it. The buffer lives until
    release() or the end of the run."""
    import tuna_gb300 as T
    dt = np.dtype(dtype)
    if like is not None:
        like = np.ascontiguousarray(like).view(dt).ravel()
        n = like.size
    hb = T.HostBuffer(max(1, n) * dt.itemsize)
    a = hb.array(dt, n)
    _HOST_BUFS.append((hb, a))
    if like is not None:
        a[:] = like
    return a


def release(*arrays) -> None:
    """Free the host memory of arrays made by host_array (not used afterwards)."""
    for a in arrays:
        for i, (hb, b) in enumerate(_HOST_BUFS):
            if b is a:
                hb.close()
                del _HOST_BUFS[i]
                break


def _pinned_copy(a):
    return host_array(0, np.uint8, like=np.asarray(a, dtype=np.uint8))


def batched_vs_plain(ctx, n_samples: int, scale: float):
    """The 2,000-sample mix, counted sample by sample through tg_count_seq (the
    plain path) and all at once through tg_count_batch; same pairs required.
    Samples go to tg_count_batch in calls of at most 8 Gbp, so that one call's
    pairs fit a reused host buffer (one call up to the 0.02 scale); inside a
    call the library counts runs of samples that fit the device."""
    import ctypes
    import tuna_gb300 as T
    from tuna_gb300 import synth
    plan = synth.batch_plan(n_samples, scale=scale)
    seqs = [_pinned_copy(synth.fastq_sequence_stream(synth.batch_sample_fastq(s, i))) for i, s in enumerate(plan)]
    bases = int(sum(s.size for s in seqs))
    L = T.library()
    o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
    cap_one = max(s.size for s in seqs)
    k1, c1 = host_array(cap_one, np.uint64), host_array(cap_one, np.uint32)
    n_out = ctypes.c_uint64()
    st = T._Stats()

    def plain(i):
        rc = L.tg_count_seq(ctx.h, ctypes.byref(o), ctypes.c_void_p(seqs[i].ctypes.data), seqs[i].size,
                            ctypes.c_void_p(k1.ctypes.data), ctypes.c_void_p(c1.ctypes.data), cap_one,
                            ctypes.byref(n_out), ctypes.byref(st))
        ctx.check(rc)
        return int(n_out.value)

    plain(0)  # warm
    t0 = time.perf_counter()
    per_plain = [plain(i) for i in range(len(seqs))]
    t_plain = time.perf_counter() - t0
    budget = 8_000_000_000  # bases per call
    runs, cur, acc = [], [], 0
    for i, sq in enumerate(seqs):
        if cur and acc + sq.size > budget:
            runs.append(cur)
            cur, acc = [], 0
        cur.append(i)
        acc += int(sq.size)
    runs.append(cur)
    calls = []
    for r in runs:
        ptrs = (ctypes.c_void_p * len(r))(*[seqs[i].ctypes.data for i in r])
        lens = (ctypes.c_size_t * len(r))(*[int(seqs[i].size) for i in r])
        # the pairs' count, from a call with no room (TG_ERR_ARG with n_out set)
        rc = L.tg_count_batch(ctx.h, ctypes.byref(o), len(r), ptrs, lens, None, None, None, 0,
                              ctypes.byref(n_out), ctypes.byref(st))
        cap_r = int(n_out.value) + 1024 if rc == 1 else int(sum(lens))
        calls.append((r, ptrs, lens, cap_r, np.zeros(len(r) + 1, dtype=np.uint64)))
    cap = max(c[3] for c in calls)
    kb, cb = host_array(cap, np.uint64), host_array(cap, np.uint32)

    def run_call(c):
        r, ptrs, lens, cap_r, off = c
        rc = L.tg_count_batch(ctx.h, ctypes.byref(o), len(r), ptrs, lens, ctypes.c_void_p(kb.ctypes.data),
                              ctypes.c_void_p(cb.ctypes.data), ctypes.c_void_p(off.ctypes.data), cap,
                              ctypes.byref(n_out), ctypes.byref(st))
        ctx.check(rc)

    def batch():
        for c in calls:
            run_call(c)

    batch()  # warm
    per_batch = [0] * len(seqs)
    for r, _, _, _, off in calls:
        for j, i in enumerate(r):
            per_batch[i] = int(off[j + 1] - off[j])
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        batch()
        ts.append(time.perf_counter() - t0)
    t_batch = statistics.median(ts)
    same_sizes = per_batch == per_plain
    # bit-exact against the oracle on 12 samples across the size range: the
    # digest of the sample's range of its batch call equals the oracle's digest
    # of that sample counted alone (and the plain path's, on the same samples)
    from oracle import oracle as O
    order = np.argsort([s.size for s in seqs])
    picks = sorted(set(int(order[int(q * (len(seqs) - 1))]) for q in np.linspace(0, 1, 12)))
    exact, checked = True, 0
    for c in calls:
        mine = [(j, i) for j, i in enumerate(c[0]) if i in picks]
        if not mine:
            continue
        run_call(c)  # this call's pairs back in kb/cb
        off = c[4]
        for j, i in mine:
            lo, hi = int(off[j]), int(off[j + 1])
            got = O.digest_pairs(kb[lo:hi].reshape(-1, 1), cb[lo:hi], 31, threads=os.cpu_count() or 1)
            want, _ = O.digest_stream(seqs[i], 31, 21, 16, threads=os.cpu_count() or 1)
            n = plain(i)
            alone = O.digest_pairs(k1[:n].reshape(-1, 1), c1[:n], 31)
            exact &= got == want == alone
            checked += 1
    release(k1, c1, kb, cb, *seqs)
    return {"workload": f"{len(seqs)} samples, genome sizes log-uniform 10 kbp - 50 Mbp scaled by {scale:g} "
                        f"(so {max(1000, 10_000 * scale) / 1e3:g} kbp floor - {50e6 * scale / 1e3:g} kbp), "
                        f"150 bp reads at 5-50x, 0.3-1% errors, k=31 m=21",
            "samples": len(seqs), "bases": bases,
            "plain_gbases_s": bases / t_plain / 1e9, "batched_gbases_s": bases / t_batch / 1e9,
            "speedup": t_plain / t_batch, "plain_s": t_plain, "batched_s": t_batch,
            "batch_calls": len(calls), "max_call_bases": budget,
            "api": "tg_count_seq per sample vs tg_count_batch (calls of at most 8 Gbp), "
                   "pinned host buffers, results in host memory",
            "same_pairs_per_sample": bool(same_sizes), "oracle_checked_samples": checked,
            "bit_exact_checked_samples": bool(exact)}


def output_drain(ctx, dev, n_stream: int):
    """Device formatting of every pair of the 3.1 Gbp job (tg_job_drain) into a
    sink that only counts bytes: TSV and KFF entries."""
    import ctypes
    import tuna_gb300 as T
    L = T.library()
    o = T._JobOpts(K, M, NPARTS, 1, (1 << 64) - 1, 0, 0)
    j = ctypes.c_void_p()
    ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
    out = {}
    try:
        ctx.check(L.tg_job_feed_seq_device(j, ctypes.c_void_p(dev.data_ptr()), n_stream))
        ctx.check(L.tg_job_run(j))
        n = int(L.tg_job_result_size(j))
        tot = [0]

        def sink(_data, nbytes, _np, _u):
            tot[0] += nbytes
            return 0

        cb = T._SINK(sink)
        for fmt, name in ((0, "tsv"), (1, "kff")):
            ctx.check(L.tg_job_drain(j, fmt, cb, None))  # warm (buffers)
            tot[0] = 0
            t0 = time.perf_counter()
            ctx.check(L.tg_job_drain(j, fmt, cb, None))
            t = time.perf_counter() - t0
            out[name] = {"seconds": t, "bytes": tot[0], "gbytes_s": tot[0] / t / 1e9, "mpairs_s": n / t / 1e6}
    finally:
        L.tg_job_end(j)
    out["pairs"] = n
    out["api"] = ("tg_job_drain (include/tuna_gpu.h): formatted on the device in 2^20-pair batches, "
                  "copied to pinned host buffers, handed to a sink that counts bytes")
    return out


def large_k(ctx, scale: float, steps: int, parity_cpu: bool = True):
    """The k=63 read set: a seeded 100 Mbp genome with 20% repeats (1 kbp
    families, 5% divergence), 150 bp reads at 30x (3 Gbp), 0.5% substitutions;
    k=63 m=21, ci=2 cx=10000. End to end from the FASTQ bytes (tg_count_fastx),
    and the device-resident step; then the KFF drain."""
    import ctypes
    import torch
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq, meta = synth.large_k_reads(scale=scale)
    L = T.library()
    k, m, ci, cx = meta["k"], meta["m"], meta["ci"], meta["cx"]
    bases = meta["reads"] * 150
    dev = torch.from_numpy(fq).cuda()
    o = T._JobOpts(k, m, 16, ci, cx, 0, 0)
    # device-resident: FASTQ bytes already in HBM, lexed and counted
    res, _ = ctx.run(k, m, dev_fastx=dev.data_ptr(), dev_len=int(fq.size), ci=ci, cx=cx, want_results=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        res, _ = ctx.run(k, m, dev_fastx=dev.data_ptr(), dev_len=int(fq.size), ci=ci, cx=cx, want_results=False)
    t_dev = (time.perf_counter() - t0) / steps
    st = res.stats
    n_out = int(st["out"])
    dres, _ = ctx.run(k, m, dev_fastx=dev.data_ptr(), dev_len=int(fq.size), ci=ci, cx=cx, want_results=False,
                      digest=True)
    del dev
    cpu_dg = None
    if parity_cpu:
        from oracle import oracle as O
        cpu_dg, _ = O.digest_stream(fq, k, m, 64, ci, cx, threads=os.cpu_count() or 1, fastx=True)
    parity = parity_against(dres.digest, fq, "bench_large_k63_m21", cpu_dg)
    h_in = host_array(0, np.uint8, like=fq)
    cap = n_out + 1024
    h_keys = host_array(cap * 2, np.uint64)
    h_cnt = host_array(cap, np.uint32)
    nout = ctypes.c_uint64()
    sts = T._Stats()

    def step():
        ctx.check(L.tg_count_fastx(ctx.h, ctypes.byref(o), ctypes.c_void_p(h_in.ctypes.data), h_in.size,
                                   ctypes.c_void_p(h_keys.ctypes.data), ctypes.c_void_p(h_cnt.ctypes.data), cap,
                                   ctypes.byref(nout), ctypes.byref(sts)))

    step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    t_e2e = (time.perf_counter() - t0) / steps
    from oracle import oracle as O
    e2e_dg = O.digest_pairs(h_keys[: int(nout.value) * 2].reshape(-1, 2), h_cnt[: int(nout.value)], k,
                            threads=os.cpu_count() or 1)
    parity["e2e_fastx_digest_same"] = e2e_dg == dres.digest
    parity["ok"] = parity["ok"] and parity["e2e_fastx_digest_same"]
    # the KFF file body of this result
    tot = [0]

    def sink(_d, nbytes, _np, _u):
        tot[0] += nbytes
        return 0

    cb = T._SINK(sink)
    j = ctypes.c_void_p()
    ctx.check(L.tg_job_begin(ctx.h, ctypes.byref(o), ctypes.byref(j)))
    try:
        ctx.check(L.tg_job_feed_fastx(j, ctypes.c_void_p(h_in.ctypes.data), h_in.size))
        ctx.check(L.tg_job_run(j))
        t0 = time.perf_counter()
        ctx.check(L.tg_job_drain(j, 1, cb, None))
        t_kff = time.perf_counter() - t0
    finally:
        L.tg_job_end(j)
    release(h_in, h_keys, h_cnt)
    return {"workload": f"{meta['genome'] / 1e6:.0f} Mbp genome, 20% repeats (1 kbp families, 5% divergence), "
                        f"{meta['reads']} reads of 150 bp (30x), 0.5% substitutions; k=63 m=21 ci=2 cx=10000",
            "bases": bases, "fastq_bytes": int(fq.size),
            "device_gbases_s": bases / t_dev / 1e9, "device_ms": t_dev * 1e3,
            "e2e_gbases_s": bases / t_e2e / 1e9, "e2e_ms": t_e2e * 1e3,
            "kmers": int(st["kmers"]), "distinct": int(st["distinct"]), "out": n_out,
            "group_load_pct": int(st["group_load_pct"]),
            "parts_ms": {f: float(st[f]) for f in ("lex_ms", "pack_ms", "phase1_ms", "phase2_keys_ms",
                                                     "phase2_count_ms")},
            "kff_drain_s": t_kff, "kff_bytes": tot[0], "parity": parity,
            "api": "device: tg_job_feed_fastx_device + tg_job_run; e2e: tg_count_fastx from pinned FASTQ bytes, "
                   "pairs to pinned host buffers"}


def passes_section(dev, n_stream: int, kmers: int, steps: int):
    """The 3.1 Gbp job on a context whose memory budget holds a quarter of its
    phase-2 keys and pairs: phase 2 in passes over ranges of bins, each pass's
    pairs copied to host memory."""
    import torch
    import tuna_gb300 as T
    per_key = 2 * 8 + 4 + 24
    budget = kmers * per_key // 4
    with T.Context(torch.cuda.current_device(), hbm_budget=budget) as c2:
        r, _ = c2.run(K, M, dev_seq=dev.data_ptr(), dev_len=n_stream, n_parts=NPARTS, want_results=False)
        t0 = time.perf_counter()
        for _ in range(steps):
            r, _ = c2.run(K, M, dev_seq=dev.data_ptr(), dev_len=n_stream, n_parts=NPARTS, want_results=False)
        t = (time.perf_counter() - t0) / steps
    st = r.stats
    return {"budget_bytes": budget, "passes": int(st["phase2_passes"]), "ms_per_step": t * 1e3,
            "gbases_s": n_stream / t / 1e9, "out": int(st["out"]),
            "phase2_ms": st["phase2_ms"], "d2h_ms": st["d2h_ms"],
            "api": "tg_ctx_opts.hbm_budget_bytes; device-resident input, every pass's pairs copied to host memory"}


def small_reads(ctx, steps: int):
    """The small read set: a seeded 4.6 Mbp genome (i.i.d., GC 50 %), 150 bp reads
    from both strands at 30x (138 Mbp), 0.5 % substitutions, 0.01 % N, as FASTQ;
    k=31 m=21. End to end from the FASTQ bytes (tg_count_fastx), and the CPU
    reference path (the oracle port) on the same bytes with all host cores."""
    import ctypes
    import torch
    import tuna_gb300 as T
    from oracle import oracle as O
    from tuna_gb300 import synth
    fq, meta = synth.reads_workload(scale=1.0, seed=1)
    bases = int(meta["reads"]) * 150
    L = T.library()
    h = host_array(0, np.uint8, like=fq)
    cap = bases
    hk = host_array(cap, np.uint64)
    hc = host_array(cap, np.uint32)
    o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
    n = ctypes.c_uint64()
    st = T._Stats()

    def step():
        ctx.check(L.tg_count_fastx(ctx.h, ctypes.byref(o), ctypes.c_void_p(h.ctypes.data), h.size,
                                   ctypes.c_void_p(hk.ctypes.data), ctypes.c_void_p(hc.ctypes.data), cap,
                                   ctypes.byref(n), ctypes.byref(st)))

    for _ in range(3):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    t = (time.perf_counter() - t0) / steps
    cores = os.cpu_count() or 1
    O.count_fastx(fq[:1_000_000], 31, 21, threads=cores)  # load, warm
    c0 = time.perf_counter()
    ref = O.count_fastx(fq, 31, 21, threads=cores)
    tc = time.perf_counter() - c0
    got = O.digest_pairs(hk[: int(n.value)].reshape(-1, 1), hc[: int(n.value)], 31, threads=cores)
    parity = parity_against(got, fq, "scale_reads_k31_m21", O.digest_pairs(ref.keys, ref.counts, 31))
    release(h, hk, hc)
    return {"workload": "4.6 Mbp genome, 920 k reads of 150 bp (30x, both strands), 0.5 % substitutions, "
                        "0.01 % N, FASTQ; k=31 m=21", "bases": bases, "fastq_bytes": int(fq.size),
            "e2e_gbases_s": bases / t / 1e9, "e2e_ms": t * 1e3, "distinct": int(n.value),
            "cpu_port_gbases_s": bases / tc / 1e9, "cpu_port_s": tc, "cpu_cores": cores,
            "same_distinct": int(n.value) == len(ref), "parity": parity,
            "api": "tg_count_fastx from pinned FASTQ bytes; CPU: the oracle port (tor_count_fastx)"}


def gz_input(ctx, fasta: np.ndarray, mbytes: float = 300.0):
    """Reading gzip input on the host (tg_read_input): a BGZF file inflated on
    1 and on all host threads, and the same bytes as one gzip member (one
    stream, as the reference's GzInput reads every .gz file). Then the whole
    path from a file (tg_job_feed_file: reading and inflating on host threads,
    H2D, lexing on the device, both phases; the pairs' digest on the device,
    which must equal the plain file's), from the BGZF file and from the same
    FASTA uncompressed."""
    import gzip
    import zlib
    from concurrent.futures import ThreadPoolExecutor
    import tuna_gb300 as T
    raw = fasta[: int(mbytes * 1e6)].tobytes()
    blk = 65280

    def member(i):
        chunk = raw[i:i + blk]
        c = zlib.compressobj(1, zlib.DEFLATED, -15)
        payload = c.compress(chunk) + c.flush()
        bsize = 18 + len(payload) + 8
        return (b"\x1f\x8b\x08\x04\x00\x00\x00\x00\x00\xff\x06\x00BC\x02\x00" + (bsize - 1).to_bytes(2, "little")
                + payload + zlib.crc32(chunk).to_bytes(4, "little") + len(chunk).to_bytes(4, "little"))

    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        bg = b"".join(ex.map(member, range(0, len(raw), blk)))
    bg += bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")
    d = tempfile.mkdtemp()
    p_bg, p_one = os.path.join(d, "a.fa.gz"), os.path.join(d, "b.fa.gz")
    with open(p_bg, "wb") as f:
        f.write(bg)
    with open(p_one, "wb") as f:
        f.write(gzip.compress(raw, compresslevel=1))
    res = {"bytes": len(raw), "bgzf_bytes": len(bg)}
    cores = os.cpu_count() or 1
    for name, path, th in (("bgzf_1_thread", p_bg, 1), ("bgzf_all_threads", p_bg, cores), ("one_member", p_one, cores)):
        T.read_input(path, th, cap=len(raw) + 1024)  # page cache warm
        t0 = time.perf_counter()
        got = T.read_input(path, th, cap=len(raw) + 1024)
        t = time.perf_counter() - t0
        assert got == raw
        res[name] = {"seconds": t, "gbytes_s": len(raw) / t / 1e9, "threads": th}
    p_plain = os.path.join(d, "c.fa")
    with open(p_plain, "wb") as f:
        f.write(raw)
    dg = {}
    for name, path in (("count_from_plain_file", p_plain), ("count_from_bgzf_file", p_bg)):
        ctx.run(K, M, files=[path], n_parts=NPARTS, want_results=False)  # page cache, buffers
        t0 = time.perf_counter()
        r, _ = ctx.run(K, M, files=[path], n_parts=NPARTS, want_results=False, digest=True)
        t = time.perf_counter() - t0
        dg[name] = r.digest
        res[name] = {"seconds": t, "gbases_s": int(r.stats["bases"]) / t / 1e9, "bases": int(r.stats["bases"]),
                     "pairs": len(r) if r.keys is not None else int(r.stats["out"])}
    res["count_from_file_digests_same"] = dg["count_from_plain_file"] == dg["count_from_bgzf_file"]
    for p in (p_bg, p_one, p_plain):
        os.remove(p)
    os.rmdir(d)
    res["api"] = ("tg_read_input (include/tuna_gpu.h), the reading step of tg_job_feed_file; "
                  "count_from_*: tg_job_feed_file + tg_job_run, pairs left on the device (digest)")
    return res


def served(seconds: float, scale: float, pool_size: int = 48, burst_rate: float = 400.0,
           burst_seconds: float = 4.0):
    """Poisson arrivals at 50 requests/s replayed in real time against the
    continuous-batching server; latency from arrival to result in host memory.
    Request sizes follow the configured distribution (log-normal, median 20 Mbp
    x scale, sigma 1.5, cap 2 Gbp x scale); the replay reuses a pool of
    `pool_size` generated requests (one third per k), the i-th arrival taking
    the next pooled request of its k. Answers are dropped as they arrive, so the
    server's result slabs are recycled. Then a burst: `burst_rate` requests/s
    for `burst_seconds` (more bases than the device counts in that time), which
    queues requests while batches run, so that they merge."""
    import threading
    from tuna_gb300 import synth
    from tuna_gb300.serve import Server
    plan = synth.served_plan(50.0, seconds, scale=scale)
    by_k = {}
    for i, r in enumerate(plan[: max(pool_size, 1) * 4]):
        lst = by_k.setdefault(r.k, [])
        if len(lst) < max(1, pool_size // 3):
            lst.append((r, _pinned_copy(synth.fastq_sequence_stream(synth.request_fastq(r, i)))))

    def replay_of(p):
        nxt = {k: 0 for k in by_k}
        out = []
        for r in p:
            lst = by_k.get(r.k) or next(iter(by_k.values()))
            pr, seq = lst[nxt.get(r.k, 0) % len(lst)]
            nxt[r.k] = nxt.get(r.k, 0) + 1
            out.append((r.arrival_s, pr.k, pr.m, seq))
        return out

    def run(srv, replay, length_s):
        lat, done_t = [], []
        mu = threading.Lock()
        left = threading.Semaphore(0)

        def record(f):
            a = f.result()
            with mu:
                lat.append(a.latency_s * 1e3)
                done_t.append(a.done)
            left.release()

        srv.batches = 0
        srv.batch_sizes.clear()
        bases = 0
        t0 = time.perf_counter()
        for arr, k, m, seq in replay:
            dt = t0 + arr - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            srv.submit(seq, k, m).add_done_callback(record)
            bases += int(seq.size)
        for _ in replay:
            left.acquire()
        t_end = max(done_t)
        sizes = list(srv.batch_sizes)
        lat_a = np.array(lat)
        hist = {}
        for n in sizes:
            hist[str(n)] = hist.get(str(n), 0) + 1
        return {"requests": len(replay), "bases": bases, "p50_ms": float(np.percentile(lat_a, 50)),
                "p99_ms": float(np.percentile(lat_a, 99)), "max_ms": float(lat_a.max()),
                "offered_gbases_s": bases / max(length_s, 1e-9) / 1e9,
                "gbases_s": bases / (t_end - t0) / 1e9, "batches": len(sizes),
                "requests_per_batch_mean": float(np.mean(sizes)) if sizes else 0.0,
                "requests_per_batch_hist": dict(sorted(hist.items(), key=lambda kv: int(kv[0])))}

    with Server(0, workers=2) as srv:
        for f in [srv.submit(by_k[k][0][1], k, by_k[k][0][0].m) for k in by_k for _ in range(2)]:
            f.result()  # warm both workers
        res = run(srv, replay_of(plan), seconds)
        burst = run(srv, replay_of(synth.served_plan(burst_rate, burst_seconds, seed=29, scale=scale)),
                    burst_seconds)
    n_pool = sum(len(v) for v in by_k.values())
    res = {"workload": f"Poisson 50 req/s for {seconds:g} s, sizes log-normal median {20 * scale:g} Mbp "
                       f"(sigma 1.5, cap {2000 * scale:g} Mbp), reads 100-250 bp at 0.5% error, "
                       f"k in {{21, 25, 31}}; {n_pool} generated requests replayed", **res}
    burst["workload"] = (f"Poisson {burst_rate:g} req/s for {burst_seconds:g} s, the same sizes and pool "
                         f"(more bases than the device counts in that time: requests queue and merge)")
    res["burst"] = burst
    res["workers"] = 2
    res["api"] = "tuna_gb300.serve.Server over the job API (several samples per job), results in page-locked host memory"
    return res


# ------------------------------------------------------------------ reference arm
def rank_barrier(world: int) -> None:
    """Barrier across the replicas (no-op for one process)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def rank_max(x: float, world: int, device: str) -> float:
    """The maximum of x over the replicas: a step's time is the slowest rank's."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank: int):
    """The reference arm: the CPU path (the oracle port of the reference's
    pipeline; the reference's own sources are not on this host) on all host
    cores, on the same assembly bytes as the GB300 arm. Each step counts the
    first --ref-mbp Mbp of it, pre-split into one shard per core, so that the
    whole --steps/--warmup run stays within a few minutes; value = those bases
    / the median step time."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    stream_h, bases, _, _ = workload(args.scale, want_fasta=False)
    n_stream = int(stream_h.size)
    sample = cpu_sample(stream_h, args.ref_mbp, threads)
    del stream_h
    base = time_cpu(threads, sample, steps=args.steps, warmup=args.warmup)
    v = base["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "ms_per_step": base["seconds"] * 1e3,  # median over the timed steps
            "config": main_config(bases, n_stream, args.gpus),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": base["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference CPU path, restated in C (oracle/tuna_oracle.c, pinned to the reference's "
                    "outputs by digest at the full 3.1 Gbp size); the reference sources are not on the GPU host"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GB300 arm
def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    t_start = time.perf_counter()
    import numpy as np
    import torch
    import tuna_gb300 as T
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    def barrier():
        rank_barrier(world)

    def max_over_ranks(x: float) -> float:
        return rank_max(x, world, "cuda")

    stream_h, bases, lens, fasta_h = workload(args.scale, want_fasta=True)
    dev = torch.from_numpy(stream_h).to(f"cuda:{local}")
    ctx = T.Context(local, autotune=not args.no_autotune)  # the first warm-up step times the group sizes
    ext = torch.cuda.ExternalStream(ctx.stream_ptr, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def step():
        r, _ = ctx.run(K, M, dev_seq=dev.data_ptr(), dev_len=dev.numel(), n_parts=NPARTS, want_results=False)
        return r.stats

    for _ in range(args.warmup):
        st = step()
    barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    launches = 0
    kern = {"pack": [], "cut": [], "keys": [], "count": [], "phase1": [], "phase2": []}
    for _ in range(args.steps):
        st = step()
        launches += int(st["gpu_launches"])
        kern["pack"].append(st["pack_ms"])
        kern["cut"].append(st["phase1_cut_ms"])
        kern["keys"].append(st["phase2_keys_ms"])
        kern["count"].append(st["phase2_count_ms"])
        kern["phase1"].append(st["phase1_ms"])
        kern["phase2"].append(st["phase2_ms"])
    e1.record(ext)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    value = bases * world / (ms / 1e3) / 1e9

    # ---- key-level parity of the full-size result: the device digest of its
    # pairs against the reference's (same input bytes) and the oracle port's
    dres, _ = ctx.run(K, M, dev_seq=dev.data_ptr(), dev_len=dev.numel(), n_parts=NPARTS, want_results=False,
                      digest=True)
    parity_full = None
    if rank == 0:
        cpu_dg, cpu_s = None, None
        if not args.no_parity_cpu:
            from oracle import oracle as O
            c0 = time.perf_counter()
            cpu_dg, _ = O.digest_stream(stream_h, K, M, NPARTS, threads=os.cpu_count() or 1)
            cpu_s = time.perf_counter() - c0
        parity_full = parity_against(dres.digest, fasta_h, "bench_rep_fasta_k31_m23", cpu_dg)
        parity_full["oracle_seconds"] = cpu_s
        parity_full["oracle_threads"] = os.cpu_count() or 1
        kmers_expected = sum(max(0, L - K + 1) for L in lens)
        parity_full["kmers"] = int(st["kmers"])
        parity_full["kmers_expected"] = kmers_expected
        parity_full["ok"] = parity_full["ok"] and dres.digest["count_sum"] == int(st["kmers"]) == kmers_expected

    # ---- roofline of the dominant kernel (algorithmic bytes / CUDA-event time)
    peak, peak_kind = load_peaks()
    avg = {k2: statistics.mean(v) for k2, v in kern.items()}
    recs = st["superkmers"]
    n_stream = int(dev.numel())
    rec_bases = st["kmers"] + recs * (K - 1)
    alg = {
        "cut": n_stream / 4 + n_stream / 8 + 8 * recs,            # packed + validity in, descriptors out
        "keys": 8 * recs + rec_bases / 4 + 8 * st["kmers"],       # descriptors + record bases in, keys out
        "count": 8 * st["kmers"] + st["out"] * 12,                # keys in, (key, count) out
        "pack": n_stream + n_stream / 4 + n_stream / 8,           # ASCII in, packed + validity out
    }
    dom = max(("cut", "keys", "count", "pack"), key=lambda x: avg[x])
    achieved = alg[dom] / (avg[dom] / 1e3) / 1e9
    cut_name = "k_cut_fixed" if (K, M) in ((31, 21), (31, 23), (21, 17), (25, 21)) else "k_cut_seq"
    kernel_names = {"cut": cut_name, "keys": "k_scan+k_plan+k_keys", "count": "k_count", "pack": "k_pack"}
    # phase 1 against the reference's algorithmic bytes B1 = N/4 + record bytes (~1.82 B/base)
    ref_record_bytes = 2 * recs + (st["kmers"] + recs * (K - 1)) / 4
    b1 = bases / 4 + ref_record_bytes
    p1_gbs = b1 / (avg["phase1"] / 1e3) / 1e9
    # phase 2 against the reference's algorithmic bytes B2 = record bytes read once +
    # one (key, u32 count) pair written per distinct k-mer (no key array round trip)
    b2 = ref_record_bytes + int(st["distinct"]) * (8 * ((K + 32) // 32) + 4)
    p2_gbs = b2 / (avg["phase2"] / 1e3) / 1e9
    traffic, traffic_source = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if dom in tj:
            traffic = tj[dom].get("bytes_per_launch_full_size")
            traffic_source = tj[dom].get("source")

    # ---- end to end through the C ABI: pinned host input -> counts in pinned host memory
    e2e = None
    if not args.no_e2e:
        n_out_cap = int(st["out"]) + 1024
        W = 1
        # inputs and outputs in the library's page-locked host memory (tg_host_alloc)
        h_in = host_array(0, np.uint8, like=stream_h)
        h_keys = host_array(n_out_cap * W, np.uint64)
        h_cnt = host_array(n_out_cap, np.uint32)
        L = T.library()
        import ctypes
        o = T._JobOpts(K, M, NPARTS, 1, (1 << 64) - 1, 0, 0)
        nout = ctypes.c_uint64()
        sts = T._Stats()

        def e2e_step(fn, h):
            rc = fn(ctx.h, ctypes.byref(o), ctypes.c_void_p(h.ctypes.data), h.size,
                    ctypes.c_void_p(h_keys.ctypes.data), ctypes.c_void_p(h_cnt.ctypes.data),
                    n_out_cap, ctypes.byref(nout), ctypes.byref(sts))
            ctx.check(rc)

        def timed(fn, h):
            nonlocal launches
            e2e_step(fn, h)  # warm
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            parts = {"h2d_ms": 0.0, "lex_ms": 0.0, "pack_ms": 0.0, "phase1_ms": 0.0, "phase2_ms": 0.0, "d2h_ms": 0.0}
            for _ in range(args.steps):
                e2e_step(fn, h)
                launches += int(sts.gpu_launches)
                for k2 in parts:
                    parts[k2] += getattr(sts, k2) / args.steps
            torch.cuda.synchronize()
            return max_over_ranks((time.perf_counter() - t0) / args.steps), parts

        # the host link alone: event-timed H2D of the same buffer (first and third copy)
        d_tmp = torch.empty(h_in.size, dtype=torch.uint8, device=f"cuda:{local}")
        link = []
        for _ in range(3):
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record()
            d_tmp.copy_(torch.from_numpy(h_in), non_blocking=True)
            c1.record()
            c1.synchronize()
            link.append(h_in.size / (c0.elapsed_time(c1) / 1e3) / 1e9)
        link_h2d_gbs = link[-1]
        del d_tmp
        t_str, parts_str = timed(L.tg_count_seq, h_in)
        e2e_stream = {"value": bases * world / t_str / 1e9, "unit": UNIT, "ms_per_step": t_str * 1e3,
                      "h2d_bytes_per_step": int(h_in.size), "d2h_bytes_per_step": int(nout.value) * (8 * W + 4),
                      "api": "tg_count_seq (include/tuna_gpu.h), pinned host buffers, input the parsed stream",
                      "parts_ms": parts_str}
        from oracle import oracle as O

        def host_digest():
            nn = int(nout.value)
            return O.digest_pairs(h_keys[:nn].reshape(-1, 1), h_cnt[:nn], K, threads=os.cpu_count() or 1)

        e2e_stream["digest_same_as_device"] = host_digest() == dres.digest
        release(h_in)
        h_fa = host_array(0, np.uint8, like=fasta_h)
        t_e2e, parts_fx = timed(L.tg_count_fastx, h_fa)
        e2e = {"value": bases * world / t_e2e / 1e9, "unit": UNIT, "ms_per_step": t_e2e * 1e3,
               "h2d_bytes_per_step": int(h_fa.size), "d2h_bytes_per_step": int(nout.value) * (8 * W + 4),
               "api": "tg_count_fastx (include/tuna_gpu.h): 60-column FASTA bytes in page-locked host memory "
                      "(tg_host_alloc), lexed on the device; pairs back in page-locked host memory",
               "parts_ms": parts_fx, "link_h2d_gbs": link_h2d_gbs, "link_h2d_gbs_first_copy": link[0],
               "stream": e2e_stream}
        e2e["digest_same_as_device"] = host_digest() == dres.digest
        if parity_full is not None:
            parity_full["e2e_digests_same"] = e2e["digest_same_as_device"] and e2e_stream["digest_same_as_device"]
            parity_full["ok"] = parity_full["ok"] and parity_full["e2e_digests_same"]
        release(h_fa, h_keys, h_cnt)

    section_s = {"main": time.perf_counter() - t_start}

    def section(name, fn, *a, **kw):
        t = time.perf_counter()
        r = fn(*a, **kw)
        section_s[name] = time.perf_counter() - t
        return r

    small = None
    if rank == 0 and not args.no_small:
        small = section("small_reads", small_reads, ctx, args.steps)
    gz = None
    if rank == 0 and not args.no_gz and fasta_h is not None:
        gz = section("gz", gz_input, ctx, fasta_h)
    output = None
    if rank == 0 and not args.no_output:
        output = section("output", output_drain, ctx, dev, n_stream)
    passes = None
    if rank == 0 and not args.no_passes:
        passes = section("passes", passes_section, dev, n_stream, int(st["kmers"]), 2)
    del dev
    large = None
    if rank == 0 and not args.no_large_k:
        large = section("large_k", large_k, ctx, args.large_k_scale, max(1, min(args.steps, 3)),
                        parity_cpu=not args.no_parity_cpu)

    batched = None
    if rank == 0 and not args.no_batch:
        batched = {f"scale_{sc}": section(f"batched_{sc}", batched_vs_plain, ctx, args.batch_samples, float(sc))
                   for sc in args.batch_scales.split(",") if sc}
    serve = None
    if rank == 0 and not args.no_serve:
        serve = section("serve", served, args.serve_seconds, args.serve_scale)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = section("cpu_baseline", lambda: time_cpu(os.cpu_count() or 1,
                                                       cpu_sample(stream_h, args.cpu_mbp, os.cpu_count() or 1)))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: seeded 3.1 Gbp repetitive assembly (tuna_gb300/synth.py), "
                    "stands in for the reference's genome assemblies",
            "config": main_config(bases, n_stream, world),
            "gpu_config": {"gpu_parts": int(st["gpu_parts"]), "group_load_pct": int(st["group_load_pct"]),
                           "autotune": "off (--no-autotune): half the table" if args.no_autotune else
                           "TG_CTX_AUTOTUNE: group size timed on the first warm-up step (35/50/65 % of the table)"},
            "stats": {"kmers": int(st["kmers"]), "superkmers": int(st["superkmers"]),
                      "distinct": int(st["distinct"]), "fallback_groups": int(st["fallback_groups"]),
                      "distinct_kmers_per_s": int(st["distinct"]) / (ms / 1e3),
                      "kmer_updates_per_s": int(st["kmers"]) / (ms / 1e3)},
            "kernels_ms": {kernel_names.get(k2, k2): round(v, 4) for k2, v in avg.items()},
            "roofline": {"bound": "hbm", "kernel": kernel_names[dom],
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "algorithmic_bytes": alg[dom], "traffic": traffic, "traffic_source": traffic_source,
                         "phase1_b1_gbs": p1_gbs, "phase1_b1_frac": p1_gbs / peak,
                         "phase2_b2_gbs": p2_gbs, "phase2_b2_frac": p2_gbs / peak},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "parity": parity_full,
            "output": output,
            "small_reads": small,
            "gz": gz,
            "passes": passes,
            "large_k": large,
            "batched": batched,
            "section_seconds": {k2: round(v2, 1) for k2, v2 in section_s.items()},
            "serve": serve,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
