"""Jobs larger than the memory budget: phase 2 in passes over ranges of bins
(tg_ctx_opts.hbm_budget_bytes). Each pass materialises only its bins' keys
(k_keys keeps the records of those bins), counts them and copies its pairs to
host memory; the union of the passes is exactly the one-run result, through
the job API, the one-call entry point and the device formatter."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream(seed=3, n=3_000_000):
    from tuna_gb300 import synth
    g = synth.genome(n, seed, 0.45, fam_a=(20, 300, 0.1), div=(0.02, 0.08))
    return g


@pytest.mark.parametrize("k,m", [(31, 21), (63, 21), (25, 13)])
def test_passes_match_one_run(k, m):
    import tuna_gb300 as T
    seq = _stream()
    with T.Context(0) as big:
        want, _ = big.run(k, m, seq=seq)
        assert want.stats["phase2_passes"] == 1
    with T.Context(0, hbm_budget=24 << 20) as small:
        got, _ = small.run(k, m, seq=seq, drain=0)
    assert got.stats["phase2_passes"] > 3
    a, b = got.sorted(), want.sorted()
    assert np.array_equal(a.keys, b.keys) and np.array_equal(a.counts, b.counts)
    assert got.stats["distinct"] == want.stats["distinct"]
    assert got.formatted.count(b"\n") == len(want)
    assert T.tsv_blob(got.keys, got.counts, k) == b"".join(sorted(got.formatted.splitlines(keepends=True)))


def test_passes_one_call_and_filter():
    import tuna_gb300 as T
    seq = _stream(5, 2_000_000)
    L = T.library()
    with T.Context(0) as big:
        want, _ = big.run(31, 21, seq=seq, ci=2, cx=50)
    with T.Context(0, hbm_budget=16 << 20) as small:
        cap = len(want) + 10
        keys = np.zeros(cap, dtype=np.uint64)
        cnt = np.zeros(cap, dtype=np.uint32)
        o = T._JobOpts(31, 21, 16, 2, 50, 0, 0)
        n = ctypes.c_uint64()
        st = T._Stats()
        rc = L.tg_count_seq(small.h, ctypes.byref(o), seq.ctypes.data, seq.size, keys.ctypes.data, cnt.ctypes.data,
                            cap, ctypes.byref(n), ctypes.byref(st))
        assert rc == 0, L.tg_last_error(small.h)
        assert st.phase2_passes > 1 and n.value == len(want)
    got = T.Result(keys[: n.value].reshape(-1, 1), cnt[: n.value], {}, 31).sorted()
    w = want.sorted()
    assert np.array_equal(got.keys, w.keys) and np.array_equal(got.counts, w.counts)


def _checksum(res) -> tuple:
    """Order-independent digest of the (key, count) pairs."""
    k = res.keys[:, 0].astype(np.uint64)
    x = k ^ (res.counts.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15))
    x ^= x >> np.uint64(31)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(29)
    return len(res), int(x.sum(dtype=np.uint64)), int(res.counts.astype(np.uint64).sum())


def test_large_job_key_launches_match_passes():
    """Above 2^28 k-mers k_keys writes the keys in two launches (half of the bins
    each); passes under a budget stay below that and use one. Same pairs."""
    import tuna_gb300 as T
    seq = _stream(9, 300_000_000)
    with T.Context(0) as big:
        one, _ = big.run(31, 21, seq=seq)
        assert one.stats["kmers"] > (1 << 28) and one.stats["phase2_passes"] == 1
    with T.Context(0, hbm_budget=6 << 30) as small:
        parts, _ = small.run(31, 21, seq=seq)
        assert parts.stats["phase2_passes"] >= 2
    assert _checksum(one) == _checksum(parts)
    assert _checksum(one)[2] == one.stats["kmers"]
