"""TG_CTX_AUTOTUNE: the first job of each key width with at least 2^26 k-mers
times its counting pass at several group sizes on its own keys and keeps the
fastest for the context. The choice changes scheduling only: the pairs are the
same as with the default group size."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_same_pairs_and_cached():
    import tuna_gb300 as T
    from tuna_gb300 import synth
    seq = synth.genome(70_000_000, 13, 0.45, fam_a=(20, 300, 0.1), div=(0.02, 0.08))
    with T.Context(0) as plain:
        want, _ = plain.run(31, 21, seq=seq)
        assert want.stats["group_load_pct"] == 50 and want.stats["autotune_trials"] == 0
    with T.Context(0, autotune=True) as tuned:
        a, _ = tuned.run(31, 21, seq=seq)
        assert a.stats["kmers"] >= (1 << 26)
        assert a.stats["autotune_trials"] == 3 and a.stats["group_load_pct"] in (35, 50, 65)
        b, _ = tuned.run(31, 21, seq=seq[: len(seq) // 2])  # same key width: the cached choice
        assert b.stats["autotune_trials"] == 0 and b.stats["group_load_pct"] == a.stats["group_load_pct"]
        c, _ = tuned.run(33, 21, seq=seq)  # two-word keys: tuned on their own
        assert c.stats["autotune_trials"] == 3
    x, y = a.sorted(), want.sorted()
    assert np.array_equal(x.keys, y.keys) and np.array_equal(x.counts, y.counts)
