"""The allocation-free entry point against the regular one.

tg_count_seq_device_noalloc is for callers that may not allocate device memory
when they call in (a plugin enqueue handed its buffers and stream, a process
whose device memory belongs to another allocator). It keeps all intermediate
arrays in one fixed device array inside the library. Here it must return the
same (k-mer, count) pairs as tg_count_seq, on two calls in a row (the second
call finds the scratch array holding the first call's data).

This file is collected last so that a run stopping at the first failure has
run every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular(ctx, stream, k, m, ci=1, cx=(1 << 64) - 1):
    r, _ = ctx.run(k, m, seq=stream, ci=ci, cx=cx)
    return r.sorted()


def _noalloc(stream_h, k, m, ci=1, cx=(1 << 64) - 1):
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    L = T.library()
    d_in = torch.from_numpy(stream_h).to("cuda:0")
    W = 1 if k <= 31 else 2
    cap = int(stream_h.size) + 16
    d_keys = torch.zeros(cap * W, dtype=torch.int64, device="cuda:0")
    d_cnt = torch.zeros(cap, dtype=torch.int32, device="cuda:0")
    o = T._JobOpts(k, m, 16, ci, cx, 0, 0)
    n_out = ctypes.c_uint64()
    err = ctypes.create_string_buffer(256)
    s = torch.cuda.current_stream()
    torch.cuda.synchronize()
    rc = L.tg_count_seq_device_noalloc(ctypes.byref(o), ctypes.c_void_p(d_in.data_ptr()), d_in.numel(),
                                       ctypes.c_void_p(d_keys.data_ptr()), ctypes.c_void_p(d_cnt.data_ptr()),
                                       cap, ctypes.byref(n_out), ctypes.c_void_p(s.cuda_stream), err, 256)
    assert rc == 0, err.value.decode()
    n = int(n_out.value)
    keys = d_keys[: n * W].cpu().numpy().view(np.uint64).reshape(n, W)
    cnt = d_cnt[:n].cpu().numpy().view(np.uint32)
    return T.Result(keys, cnt, {}, k).sorted()


@pytest.mark.parametrize("k,m", [(31, 21), (63, 21), (21, 17)])
def test_noalloc_matches_regular_twice(k, m):
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g = synth.genome(200_000, 41, 0.45, fam_a=(5, 300, 0.3), div=(0.02, 0.05), micro=0.05)
    fq = synth.reads_fastq(g, 2500, 150, 0.005, 0.0005, 42)
    stream = synth.fastq_sequence_stream(fq)
    assert stream.size <= (1 << 19)
    with T.Context(0) as ctx:
        want = _regular(ctx, stream, k, m)
    for _ in range(2):
        got = _noalloc(stream, k, m)
        assert len(got) == len(want)
        assert np.array_equal(got.keys, want.keys)
        assert np.array_equal(got.counts, want.counts)


def test_noalloc_allocates_nothing_after_warmup():
    """After one warm-up call (len == 0, which reserves the scratch array on the
    device) a counting call leaves the device's free memory unchanged: it
    allocates nothing. Counting the same input twice gives the same pairs."""
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    from tuna_gb300 import synth
    L = T.library()
    o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
    n_out = ctypes.c_uint64(7)
    err = ctypes.create_string_buffer(256)
    stream = synth.fastq_sequence_stream(synth.reads_fastq(synth.genome(100_000, 5, 0.5), 2000, 150, 0.005, 0.0, 6))
    d_in = torch.from_numpy(stream).to("cuda:0")
    cap = int(stream.size)
    d_keys = torch.zeros(cap, dtype=torch.int64, device="cuda:0")
    d_cnt = torch.zeros(cap, dtype=torch.int32, device="cuda:0")
    s = torch.cuda.current_stream()

    def call(n):
        return L.tg_count_seq_device_noalloc(ctypes.byref(o), ctypes.c_void_p(d_in.data_ptr()), n,
                                             ctypes.c_void_p(d_keys.data_ptr()), ctypes.c_void_p(d_cnt.data_ptr()),
                                             cap, ctypes.byref(n_out), ctypes.c_void_p(s.cuda_stream), err, 256)

    assert call(0) == 0, err.value.decode()
    assert n_out.value == 0
    assert call(d_in.numel()) == 0, err.value.decode()  # loads the kernels this input uses
    first = (d_keys[: n_out.value].cpu().numpy().copy(), d_cnt[: n_out.value].cpu().numpy().copy())
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert call(d_in.numel()) == 0, err.value.decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    a = np.sort(first[0])
    b = np.sort(d_keys[: n_out.value].cpu().numpy())
    assert np.array_equal(a, b)


def test_noalloc_filters_and_limits():
    torch = pytest.importorskip("torch")
    import tuna_gb300 as T
    from tuna_gb300 import synth
    fq = synth.reads_fastq(synth.genome(50_000, 3, 0.5), 3000, 150, 0.005, 0.0, 4)
    stream = synth.fastq_sequence_stream(fq)
    with T.Context(0) as ctx:
        want = _regular(ctx, stream, 31, 21, ci=2, cx=9)
    got = _noalloc(stream, 31, 21, ci=2, cx=9)
    assert np.array_equal(got.keys, want.keys) and np.array_equal(got.counts, want.counts)
    # over the size limit: a clear error, nothing allocated
    L = T.library()
    big = torch.zeros((1 << 19) + 1, dtype=torch.uint8, device="cuda:0")
    o = T._JobOpts(31, 21, 16, 1, (1 << 64) - 1, 0, 0)
    n_out = ctypes.c_uint64()
    err = ctypes.create_string_buffer(256)
    rc = L.tg_count_seq_device_noalloc(ctypes.byref(o), ctypes.c_void_p(big.data_ptr()), big.numel(),
                                       None, None, 0, ctypes.byref(n_out), None, err, 256)
    assert rc == 1 and b"exceeds the no-allocation limit" in err.value
