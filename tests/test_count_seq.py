"""tg_count_seq, the one-call entry point with host buffers (the bench's end-to-end
path): its counting pass runs in waves whose pairs are copied to the caller's
buffers while later waves count. Same pairs as the job API; a buffer that is too
small gives TG_ERR_ARG with the needed size."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    from tuna_gb300 import synth
    g = synth.genome(2_000_000, 7, 0.41, fam_a=(20, 300, 0.2), div=(0.02, 0.1), micro=0.03)
    fq = synth.reads_fastq(g, 40_000, 150, 0.005, 0.0005, 11)
    return synth.fastq_sequence_stream(fq)


def _count_seq(ctx, stream, k, m, cap, pinned):
    import tuna_gb300 as T
    L = T.library()
    W = 1 if k <= 31 else 2
    if pinned:
        torch = pytest.importorskip("torch")
        h_in = torch.from_numpy(stream).pin_memory()
        keys = torch.zeros(max(cap, 1) * W, dtype=torch.int64, pin_memory=True)
        cnt = torch.zeros(max(cap, 1), dtype=torch.int32, pin_memory=True)
        p_in, p_keys, p_cnt = h_in.data_ptr(), keys.data_ptr(), cnt.data_ptr()
    else:
        h_in = np.ascontiguousarray(stream)
        keys = np.zeros(max(cap, 1) * W, dtype=np.uint64)
        cnt = np.zeros(max(cap, 1), dtype=np.uint32)
        p_in, p_keys, p_cnt = h_in.ctypes.data, keys.ctypes.data, cnt.ctypes.data
    o = T._JobOpts(k, m, 16, 1, (1 << 64) - 1, 0, 0)
    n_out = ctypes.c_uint64()
    st = T._Stats()
    rc = L.tg_count_seq(ctx.h, ctypes.byref(o), ctypes.c_void_p(p_in), int(stream.size), ctypes.c_void_p(p_keys),
                        ctypes.c_void_p(p_cnt), cap, ctypes.byref(n_out), ctypes.byref(st))
    n = int(n_out.value)
    if pinned:
        keys = keys.numpy().view(np.uint64)
        cnt = cnt.numpy().view(np.uint32)
    return rc, n, keys, cnt, st


@pytest.mark.parametrize("k,m,pinned", [(31, 21, True), (31, 21, False), (63, 21, True)])
def test_count_seq_matches_job(k, m, pinned):
    import tuna_gb300 as T
    stream = _stream()
    with T.Context(0) as ctx:
        want, _ = ctx.run(k, m, seq=stream)
        want = want.sorted()
        rc, n, keys, cnt, st = _count_seq(ctx, stream, k, m, len(want) + 7, pinned)
        assert rc == 0, T.library().tg_last_error(ctx.h)
        assert n == len(want)
        W = 1 if k <= 31 else 2
        got = T.Result(keys[: n * W].reshape(n, W), cnt[:n], {}, k).sorted()
        assert np.array_equal(got.keys, want.keys)
        assert np.array_equal(got.counts, want.counts)
        assert st.d2h_ms > 0


def test_count_seq_small_buffer():
    import tuna_gb300 as T
    stream = _stream()
    with T.Context(0) as ctx:
        want, _ = ctx.run(31, 21, seq=stream)
        rc, n, _, _, _ = _count_seq(ctx, stream, 31, 21, len(want) // 2, True)
        assert rc == 1  # TG_ERR_ARG
        assert n == len(want)
