"""Output formatting on the device (csrc/tg_format.cu, tg_job_drain) against
the same pairs formatted here: TSV lines as write_counts prints them
(src/count.hpp:180-216), KFF raw-section entries (src/kff_output.hpp:42-57:
ceil(k/4) bytes MSB-first 2-bit codes, count as u32 big-endian) and RAW
records, in the order of tg_job_result_copy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tsv(res) -> bytes:
    import tuna_gb300 as T
    if len(res) == 0:
        return b""
    lab = T.label_array(res.keys, res.k)
    return b"".join(bytes(lab[i]) + b"\t" + str(int(c)).encode() + b"\n" for i, c in enumerate(res.counts))


def _kff(res) -> bytes:
    k = res.k
    kb = (k + 3) // 4
    out = bytearray()
    for i in range(len(res)):
        v = 0
        for w in range(res.keys.shape[1] - 1, -1, -1):
            v = (v << 64) | int(res.keys[i, w])
        rec = bytearray(kb)
        for j in range(k):
            c = (v >> (2 * (k - 1 - j))) & 3
            rec[j >> 2] |= c << (6 - 2 * (j & 3))
        out += rec + int(res.counts[i]).to_bytes(4, "big")
    return bytes(out)


def _raw(res) -> bytes:
    W = res.keys.shape[1]
    rec = np.zeros(len(res), dtype=[("k", "<u8", (W,)), ("c", "<u4")])
    rec["k"] = res.keys
    rec["c"] = res.counts
    return rec.tobytes()


def _input(seed: int) -> np.ndarray:
    from tuna_gb300 import synth
    g = synth.genome(30_000, seed, 0.45)
    fq = synth.reads_fastq(g, 2_000, (60, 180), 0.01, 0.001, seed + 1)
    # a long poly-A run: counts of six digits
    return np.concatenate([fq, np.frombuffer(b"@p\n" + b"A" * 150_000 + b"\n+\n" + b"I" * 150_000 + b"\n",
                                             dtype=np.uint8)])


@pytest.mark.parametrize("k,m", [(5, 3), (21, 11), (31, 21), (32, 21), (33, 17), (63, 21)])
@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_drain_matches_pairs(k, m, fmt):
    import tuna_gb300 as T
    data = _input(k)
    with T.Context(0) as ctx:
        res, _ = ctx.run(k, m, fastx=data, drain=fmt)
    want = (_tsv, _kff, _raw)[fmt](res)
    assert res.formatted == want
    if fmt == 0:
        assert max(int(c) for c in res.counts) > 99_999


def test_drain_many_batches():
    """More pairs than one drain batch (2^20): the batches arrive in order."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    g = synth.genome(1_500_000, 5, 0.5)
    with T.Context(0) as ctx:
        res, _ = ctx.run(31, 21, seq=g, drain=0)
    assert len(res) > (1 << 20)
    lines = res.formatted.split(b"\n")[:-1]
    assert len(lines) == len(res)
    assert res.formatted == _tsv(res)
