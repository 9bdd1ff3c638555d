"""Bins far larger than a shared-memory table, with mostly distinct keys: the
retry passes (a failed group comes back as key-hash parts, as many as its
estimated distinct keys need) and, past 64 parts, the global-memory table
(k_fb_*). The input is many copies of one conserved 21-mer with a very small
canonical ntHash between random flanks: every k-mer covering the core has it
as minimizer, so they all land in one bin, and the flanks make them distinct."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _core(seed: int = 5) -> bytes:
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    best = None
    for _ in range(20000):
        c = rng.choice(acgt, 21).tobytes()
        h = O.nthash(c)
        if best is None or h < best[0]:
            best = (h, c)
    return best[1]


def _repeat_stream(n_copies: int, seed: int) -> np.ndarray:
    core = np.frombuffer(_core(), dtype=np.uint8)
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", dtype=np.uint8)
    rows = np.empty((n_copies, 40 + 21 + 40 + 1), dtype=np.uint8)
    rows[:, :40] = rng.choice(acgt, (n_copies, 40))
    rows[:, 40:61] = core
    rows[:, 61:101] = rng.choice(acgt, (n_copies, 40))
    rows[:, 101] = ord("N")
    return rows.ravel()


@pytest.mark.parametrize("n_copies,expect_fallback", [(5_000, False), (90_000, True)])
def test_heavy_bin_retries_and_fallback(n_copies, expect_fallback):
    import tuna_gb300 as T
    seq = _repeat_stream(n_copies, 17 + n_copies)
    with T.Context(0) as ctx:
        got, _ = ctx.run(31, 21, seq=seq)
    assert got.stats["heavy_groups"] >= 1
    assert (got.stats["fallback_groups"] > 0) == expect_fallback
    want = O.count_stream(seq, 31, 21, threads=8)
    assert len(got) == len(want)
    assert T.tsv_blob(got.keys, got.counts, 31) == O.tsv_blob(want)
