"""Jobs of several samples: every sample's pairs are the same as when it runs
alone (bit-exact), whatever else is in the job — uneven sizes, empty and
tiny samples, samples that share k-mers, k = 31 and k = 63, the job API and
the one-call tg_count_batch."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _samples(n, seed):
    from tuna_gb300 import synth
    rng = np.random.default_rng(seed)
    out = []
    shared = synth.genome(60_000, seed, 0.45)
    for i in range(n):
        if i % 7 == 3:
            out.append(np.zeros(0, dtype=np.uint8))                     # empty sample
            continue
        if i % 7 == 5:
            out.append(np.frombuffer(b"ACGTACGTAC\nACG", dtype=np.uint8))  # shorter than k
            continue
        glen = int(rng.integers(5_000, 200_000))
        g = shared if i % 3 == 0 else synth.genome(glen, seed * 1000 + i, 0.41, fam_a=(3, 300, 0.2),
                                                    div=(0.05, 0.1), micro=0.03)
        cov = float(rng.uniform(2, 12))
        nreads = max(1, int(glen * cov / 150))
        fq = synth.reads_fastq(g, nreads, 150, 0.005, 0.0005, seed * 7 + i)
        out.append(synth.fastq_sequence_stream(fq))
    return out


def _same(a, b):
    a, b = a.sorted(), b.sorted()
    return len(a) == len(b) and np.array_equal(a.keys, b.keys) and np.array_equal(a.counts, b.counts)


@pytest.mark.parametrize("k,m", [(31, 21), (63, 21), (21, 17)])
def test_each_sample_alone_and_in_the_mix(k, m):
    import tuna_gb300 as T
    smp = _samples(12, 5)
    with T.Context(0) as ctx:
        mix, _ = ctx.run(k, m, samples=smp)
        assert mix.samples is not None and len(mix.samples) == len(mix)
        assert int(mix.samples.max(initial=0)) < len(smp)
        for i, s in enumerate(smp):
            alone, _ = ctx.run(k, m, seq=s)
            assert _same(mix.sample(i), alone), f"sample {i}"


def test_many_small_samples():
    import tuna_gb300 as T
    from tuna_gb300 import synth
    smp = []
    for i in range(300):
        g = synth.genome(3_000 + 50 * i, 900 + i, 0.5)
        fq = synth.reads_fastq(g, 60, 150, 0.005, 0.0, 3 + i)
        smp.append(synth.fastq_sequence_stream(fq))
    with T.Context(0) as ctx:
        mix, _ = ctx.run(31, 21, samples=smp)
        for i in (0, 1, 57, 150, 299):
            alone, _ = ctx.run(31, 21, seq=smp[i])
            assert _same(mix.sample(i), alone), f"sample {i}"
        assert sum(len(ctx.run(31, 21, seq=s)[0]) for s in smp[:20]) == int((mix.samples < 20).sum())


def test_count_batch_one_call():
    import tuna_gb300 as T
    torch = pytest.importorskip("torch")
    smp = _samples(9, 8)
    with T.Context(0) as ctx:
        want, _ = ctx.run(31, 21, samples=smp)
        L = T.library()
        bufs = [torch.from_numpy(np.array(s, dtype=np.uint8)).pin_memory() if s.size else None for s in smp]
        ptrs = (ctypes.c_void_p * len(smp))(*[b.data_ptr() if b is not None else None for b in bufs])
        lens = (ctypes.c_size_t * len(smp))(*[int(s.size) for s in smp])
        cap = len(want) + 5
        keys = torch.zeros(cap, dtype=torch.int64, pin_memory=True)
        cnt = torch.zeros(cap, dtype=torch.int32, pin_memory=True)
        off = np.zeros(len(smp) + 1, dtype=np.uint64)
        o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
        n_out = ctypes.c_uint64()
        st = T._Stats()
        rc = L.tg_count_batch(ctx.h, ctypes.byref(o), len(smp), ptrs, lens, ctypes.c_void_p(keys.data_ptr()),
                              ctypes.c_void_p(cnt.data_ptr()), ctypes.c_void_p(off.ctypes.data), cap,
                              ctypes.byref(n_out), ctypes.byref(st))
        assert rc == 0, L.tg_last_error(ctx.h)
        n = int(n_out.value)
        assert n == len(want) and int(off[-1]) == n and np.all(np.diff(off.astype(np.int64)) >= 0)
        kk = keys[:n].numpy().view(np.uint64).reshape(n, 1)
        cc = cnt[:n].numpy().view(np.uint32)
        for i in range(len(smp)):
            a, b = int(off[i]), int(off[i + 1])
            assert _same(T.Result(kk[a:b], cc[a:b], {}, 31), want.sample(i)), f"sample {i}"


def test_export_needs_one_sample():
    import tuna_gb300 as T
    smp = _samples(3, 2)
    with T.Context(0) as ctx:
        with pytest.raises(T.GpuError):
            ctx.run(31, 21, samples=smp, export=True, want_results=False)


def test_count_batch_fastx_matches_alone():
    """tg_count_batch_fastx: FASTA and FASTQ files, one empty, lexed on the device
    into separate samples; each sample's pairs are its pairs alone."""
    import ctypes
    import tuna_gb300 as T
    from tuna_gb300 import synth
    files = []
    for i in range(6):
        g = synth.genome(30_000 + 10_000 * i, 300 + i, 0.45)
        if i == 3:
            files.append(np.zeros(0, dtype=np.uint8))
        elif i % 2:
            files.append(synth.fasta(g, [g.size // 2, g.size - g.size // 2]))
        else:
            files.append(synth.reads_fastq(g, 300, (100, 250), 0.005, 0.001, 70 + i))
    L = T.library()
    ptrs = (ctypes.c_void_p * len(files))(*[f.ctypes.data if f.size else None for f in files])
    lens = (ctypes.c_size_t * len(files))(*[int(f.size) for f in files])
    cap = sum(int(f.size) for f in files)
    keys = np.zeros(cap, dtype=np.uint64)
    cnt = np.zeros(cap, dtype=np.uint32)
    off = np.zeros(len(files) + 1, dtype=np.uint64)
    o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
    n = ctypes.c_uint64()
    st = T._Stats()
    with T.Context(0) as ctx:
        rc = L.tg_count_batch_fastx(ctx.h, ctypes.byref(o), len(files), ptrs, lens, keys.ctypes.data, cnt.ctypes.data,
                                    off.ctypes.data, cap, ctypes.byref(n), ctypes.byref(st))
        assert rc == 0, L.tg_last_error(ctx.h)
        for i, f in enumerate(files):
            a, b = int(off[i]), int(off[i + 1])
            if f.size == 0:
                assert a == b
                continue
            want = ctx.run(31, 21, fastx=f)[0].sorted()
            got = T.Result(keys[a:b].reshape(-1, 1).copy(), cnt[a:b].copy(), {}, 31).sorted()
            assert np.array_equal(got.keys, want.keys) and np.array_equal(got.counts, want.counts)


def _count_batch(ctx, smp, k, m, cap, fastx=False):
    import tuna_gb300 as T
    L = T.library()
    ptrs = (ctypes.c_void_p * len(smp))(*[s.ctypes.data if s.size else None for s in smp])
    lens = (ctypes.c_size_t * len(smp))(*[int(s.size) for s in smp])
    W = 1 if k <= 31 else 2
    keys = np.zeros(max(1, cap) * W, dtype=np.uint64)
    cnt = np.zeros(max(1, cap), dtype=np.uint32)
    off = np.zeros(len(smp) + 1, dtype=np.uint64)
    o = T._JobOpts(k, m, 16, 1, (1 << 64) - 1, 0, 0)
    n = ctypes.c_uint64()
    st = T._Stats()
    fn = L.tg_count_batch_fastx if fastx else L.tg_count_batch
    rc = fn(ctx.h, ctypes.byref(o), len(smp), ptrs, lens, keys.ctypes.data if cap else None,
            cnt.ctypes.data if cap else None, off.ctypes.data, cap, ctypes.byref(n), ctypes.byref(st))
    return rc, int(n.value), keys.reshape(-1, W), cnt, off, st


@pytest.mark.parametrize("k,m", [(31, 21), (63, 21)])
def test_count_batch_in_runs_of_samples(k, m):
    """A batch larger than the context's device budget runs as consecutive runs
    of samples, each run's result copy overlapping the next run's counting
    (and samples larger than a run alone, counted in passes): every sample's
    range equals its pairs alone, the offsets are consecutive, a call with no
    room reports the total, and a short buffer gets the samples that fit."""
    import tuna_gb300 as T
    smp = _samples(24, 11)
    total = sum(int(s.size) for s in smp)
    with T.Context(0) as ref, T.Context(0, hbm_budget=40 << 20) as ctx:
        want = [ref.run(k, m, seq=s)[0] for s in smp]
        n_all = sum(len(w) for w in want)
        assert total > (40 << 20) // 40 * 4  # several runs
        rc, n, keys, cnt, off, st = _count_batch(ctx, smp, k, m, 0)
        assert rc == 1 and n == n_all  # TG_ERR_ARG: no room, the count reported
        rc, n, keys, cnt, off, st = _count_batch(ctx, smp, k, m, n_all)
        assert rc == 0, T.library().tg_last_error(ctx.h)
        assert n == n_all and int(off[0]) == 0 and int(off[-1]) == n_all
        assert st.kmers == sum(int(w.stats["kmers"]) for w in want)
        for i, w in enumerate(want):
            a, b = int(off[i]), int(off[i + 1])
            got = T.Result(keys[a:b].copy(), cnt[a:b].copy(), {}, k)
            assert _same(got, w), f"sample {i}"
        # and against the oracle, sample by sample (its digest of the sample
        # counted alone on the CPU)
        from oracle import oracle as O
        for i in (0, 1, 11, 23):
            a, b = int(off[i]), int(off[i + 1])
            assert O.digest_pairs(keys[a:b], cnt[a:b], k) == O.digest_stream(smp[i], k, m, 16)[0], f"sample {i}"
        # a buffer for half the pairs: the samples that end within it are complete
        # (the order of a sample's pairs is not fixed from one call to the next)
        half = n_all // 2
        rc, n, keys2, cnt2, off2, _ = _count_batch(ctx, smp, k, m, half)
        assert rc == 1 and n == n_all and np.array_equal(off2, off)
        full = [i for i in range(len(smp)) if int(off2[i + 1]) <= half]
        assert len(full) >= 2
        for i in full:
            a, b = int(off2[i]), int(off2[i + 1])
            assert _same(T.Result(keys2[a:b].copy(), cnt2[a:b].copy(), {}, k), want[i]), f"sample {i}"


def test_count_batch_fastx_in_runs():
    """tg_count_batch_fastx under a small device budget: runs of files."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    files = []
    for i in range(10):
        g = synth.genome(40_000 + 20_000 * i, 500 + i, 0.45)
        files.append(synth.reads_fastq(g, 2_000 + 300 * i, (100, 250), 0.005, 0.001, 90 + i) if i % 2
                     else synth.fasta(g, [g.size // 3, g.size - g.size // 3]))
    with T.Context(0) as ref, T.Context(0, hbm_budget=16 << 20) as ctx:
        want = [ref.run(31, 21, fastx=f)[0] for f in files]
        n_all = sum(len(w) for w in want)
        rc, n, keys, cnt, off, _ = _count_batch(ctx, files, 31, 21, n_all, fastx=True)
        assert rc == 0 and n == n_all
        for i, w in enumerate(want):
            a, b = int(off[i]), int(off[i + 1])
            assert _same(T.Result(keys[a:b].copy(), cnt[a:b].copy(), {}, 31), w), f"file {i}"
