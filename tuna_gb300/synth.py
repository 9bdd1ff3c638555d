"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference measures on real assemblies and read sets that are not available
here; these generators stand in for them with the sizes and value
distributions of each workload:

  reads_workload   4.6 Mbp i.i.d. genome (GC 50%), 150 bp reads from both
                   strands at 30x, 0.5% substitutions, 0.01% N, Phred-30 FASTQ
  repetitive_fasta 3.1 Gbp in 24 contigs of 50-250 Mbp, GC 41%, 45% of the
                   sequence from 300 bp / 6 kbp repeat families at 10-20%
                   divergence, 3% microsatellites (1-6 bp units), 60-col FASTA
  large_k_reads    100 Mbp genome with 20% repeats (1 kbp families, 5%
                   divergence), 150 bp reads at 30x, 0.5% substitutions
  batch_samples    independent samples, genome sizes log-uniform in
                   10 kbp-50 Mbp, coverage U(5,50), error U(0.3%,1%), 150 bp
  served_requests  Poisson arrivals of count jobs, log-normal sizes (median
                   20 Mbp, sigma 1.5, capped), reads 100-250 bp at 0.5% error,
                   k in {21, 25, 31} (m = 21, or 17 for k = 21)

Every generator takes a `scale` so tests can run the same shapes small.
Byte output depends only on the seed and parameters (see csrc/synth.c).
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

from . import build as _build

_lib = None


def _L():
    global _lib
    if _lib is None:
        path = _build.synth_lib(build_if_missing=True)
        L = ctypes.CDLL(path)
        u64, u32, d, vp, i32 = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        L.synth_genome.argtypes = [vp, u64, u64, d, u32, u32, d, u32, u32, d, d, d, d, u32, u32, i32]
        L.synth_genome.restype = i32
        L.synth_reads_fastq.argtypes = [vp, u64, u64, u32, u32, d, d, u64, vp, i32]
        L.synth_reads_fastq.restype = u64
        L.synth_fasta.argtypes = [vp, vp, u32, vp]
        L.synth_fasta.restype = u64
        _lib = L
    return _lib


def _threads() -> int:
    return max(1, min(64, os.cpu_count() or 1))


def genome(length: int, seed: int, gc: float = 0.5, *, fam_a: Tuple[int, int, float] = (0, 0, 0.0),
           fam_b: Tuple[int, int, float] = (0, 0, 0.0), div: Tuple[float, float] = (0.0, 0.0),
           micro: float = 0.0, micro_len: Tuple[int, int] = (20, 200)) -> np.ndarray:
    """ASCII genome. fam_* = (n_families, family_length, fraction_of_sequence)."""
    out = np.empty(int(length), dtype=np.uint8)
    _L().synth_genome(out.ctypes.data, out.size, seed, gc,
                      fam_a[0], fam_a[1], fam_a[2], fam_b[0], fam_b[1], fam_b[2],
                      div[0], div[1], micro, micro_len[0], micro_len[1], _threads())
    return out


def reads_fastq(g: np.ndarray, n_reads: int, read_len=150, err: float = 0.005,
                n_rate: float = 0.0, seed: int = 1) -> np.ndarray:
    """FASTQ bytes of reads sampled uniformly from both strands of g."""
    lo, hi = (read_len, read_len) if isinstance(read_len, int) else read_len
    L = _L()
    n = L.synth_reads_fastq(g.ctypes.data, g.size, n_reads, lo, hi, err, n_rate, seed, None, 1)
    out = np.empty(int(n), dtype=np.uint8)
    L.synth_reads_fastq(g.ctypes.data, g.size, n_reads, lo, hi, err, n_rate, seed,
                        out.ctypes.data, _threads())
    return out


def fasta(g: np.ndarray, contig_lens) -> np.ndarray:
    lens = np.ascontiguousarray(contig_lens, dtype=np.uint64)
    assert int(lens.sum()) <= g.size
    L = _L()
    n = L.synth_fasta(g.ctypes.data, lens.ctypes.data, lens.size, None)
    out = np.empty(int(n), dtype=np.uint8)
    L.synth_fasta(g.ctypes.data, lens.ctypes.data, lens.size, out.ctypes.data)
    return out


def fastq_sequence_stream(fq: np.ndarray) -> np.ndarray:
    """The sequence lines of a well-formed 4-line FASTQ, each followed by LF.
    Any non-ACGT byte separates runs, so this is the GPU library's input."""
    nl = np.flatnonzero(fq == 10)
    starts = nl[0::4] + 1
    ends = nl[1::4] + 1
    lens = ends - starts
    idx = np.repeat(starts - np.concatenate(([0], np.cumsum(lens)[:-1])), lens) + np.arange(int(lens.sum()))
    return fq[idx]


# ---------------------------------------------------------------- workloads

def reads_workload(scale: float = 1.0, seed: int = 1) -> Tuple[np.ndarray, dict]:
    """FASTQ of the small read set; scale multiplies the genome size."""
    glen = max(1000, int(4_600_000 * scale))
    g = genome(glen, seed, 0.5)
    n_reads = int(glen * 30 / 150)
    fq = reads_fastq(g, n_reads, 150, 0.005, 0.0001, seed + 100)
    return fq, dict(k=31, m=21, ci=1, genome=glen, reads=n_reads)


def repetitive_genome(scale: float = 1.0, seed: int = 7) -> Tuple[np.ndarray, np.ndarray]:
    """Sequence and contig lengths of the 3.1 Gbp repetitive assembly."""
    total = int(3_100_000_000 * scale)
    rng = np.random.default_rng(seed)
    n = 24
    lo, hi = 50_000_000 * scale, 250_000_000 * scale
    w = rng.random(n) + 0.25
    lens = lo + (total - n * lo) * w / w.sum()
    lens = np.minimum(lens, hi).astype(np.uint64)
    lens[-1] += np.uint64(total - int(lens.sum()))
    g = genome(total, seed, 0.41, fam_a=(200, 300, 0.25), fam_b=(40, 6000, 0.20),
               div=(0.10, 0.20), micro=0.03, micro_len=(20, 200))
    return g, lens


def repetitive_fasta(scale: float = 1.0, seed: int = 7) -> Tuple[np.ndarray, dict]:
    g, lens = repetitive_genome(scale, seed)
    fa = fasta(g, lens)
    return fa, dict(k=31, m=23, n=4096, bases=int(g.size), contigs=lens.tolist())


def large_k_reads(scale: float = 1.0, seed: int = 11) -> Tuple[np.ndarray, dict]:
    glen = max(2000, int(100_000_000 * scale))
    g = genome(glen, seed, 0.5, fam_a=(100, 1000, 0.20), div=(0.05, 0.05))
    n_reads = int(glen * 30 / 150)
    fq = reads_fastq(g, n_reads, 150, 0.005, 0.0, seed + 100)
    return fq, dict(k=63, m=21, ci=2, cx=10000, genome=glen, reads=n_reads)


@dataclass
class Sample:
    genome_len: int
    coverage: float
    err: float
    fastq: Optional[np.ndarray] = None


def batch_plan(n_samples: int = 2000, seed: int = 13, scale: float = 1.0) -> List[Sample]:
    """Sample sizes of the batched workload (log-uniform 10 kbp - 50 Mbp)."""
    rng = np.random.default_rng(seed)
    lg = rng.uniform(math.log(10_000), math.log(50_000_000), n_samples)
    cov = rng.uniform(5, 50, n_samples)
    err = rng.uniform(0.003, 0.01, n_samples)
    return [Sample(max(1000, int(math.exp(x) * scale)), float(c), float(e)) for x, c, e in zip(lg, cov, err)]


def batch_sample_fastq(s: Sample, idx: int, seed: int = 13) -> np.ndarray:
    g = genome(s.genome_len, seed * 1_000_003 + idx, 0.5)
    n_reads = max(1, int(s.genome_len * s.coverage / 150))
    return reads_fastq(g, n_reads, 150, s.err, 0.0, seed * 7_000_003 + idx)


@dataclass
class Request:
    arrival_s: float
    bases: int
    k: int
    m: int


def served_plan(rate_hz: float = 50.0, duration_s: float = 600.0, seed: int = 17,
                median_bases: float = 20e6, sigma: float = 1.5, cap: float = 2e9,
                scale: float = 1.0) -> List[Request]:
    rng = np.random.default_rng(seed)
    t = 0.0
    out: List[Request] = []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > duration_s:
            break
        b = min(cap, median_bases * math.exp(sigma * rng.standard_normal()))
        k = int(rng.choice([21, 25, 31]))
        out.append(Request(t, max(2000, int(b * scale)), k, 17 if k == 21 else 21))
    return out


def request_fastq(r: Request, idx: int, seed: int = 17) -> np.ndarray:
    """Reads of 100-250 bp at 0.5% error, 20x over a genome of bases/20."""
    glen = max(1000, r.bases // 20)
    g = genome(glen, seed * 1_000_003 + idx, 0.5)
    n_reads = max(1, r.bases // 175)
    return reads_fastq(g, n_reads, (100, 250), 0.005, 0.0, seed * 7_000_003 + idx)
