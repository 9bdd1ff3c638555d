"""The serving loop (tuna_gb300/serve.py): requests of different k and sizes,
submitted from two client threads while batches are on the device; each
answer must be exactly the request's result alone."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from tuna_gb300 import synth
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(24):
        k = [21, 25, 31][i % 3]
        m = 17 if k == 21 else 21
        glen = int(rng.integers(2_000, 120_000))
        g = synth.genome(glen, 500 + i, 0.45, fam_a=(2, 300, 0.1), div=(0.05, 0.1))
        fq = synth.reads_fastq(g, max(1, glen * 8 // 175), (100, 250), 0.005, 0.0, 40 + i)
        reqs.append((synth.fastq_sequence_stream(fq), k, m))
    return reqs


def test_served_answers_match_alone():
    import tuna_gb300 as T
    from tuna_gb300.serve import Server
    reqs = _requests()
    futs = [None] * len(reqs)

    def client(idx):
        for i in idx:
            futs[i] = srv.submit(reqs[i][0], reqs[i][1], reqs[i][2])
            time.sleep(0.003)

    with Server(0, workers=2) as srv:
        th = [threading.Thread(target=client, args=(range(j, len(reqs), 2),)) for j in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        answers = [f.result(timeout=300) for f in futs]
    with T.Context(0) as ctx:
        for (seq, k, m), a in zip(reqs, answers):
            want = ctx.run(k, m, seq=seq)[0].sorted()
            got = T.Result(a.keys.copy(), a.counts.copy(), {}, k).sorted()
            assert len(got) == len(want)
            assert np.array_equal(got.keys, want.keys) and np.array_equal(got.counts, want.counts)
            assert a.latency_s >= 0
    assert max(a.batch for a in answers) >= 1


def test_served_fastq_requests_match_alone():
    """Requests given as FASTQ bytes (lexed on the device, tg_count_batch_fastx),
    mixed with stream requests of the same k: each answer is the request's
    result alone."""
    import tuna_gb300 as T
    from tuna_gb300 import synth
    from tuna_gb300.serve import Server
    reqs = []
    for i in range(10):
        g = synth.genome(20_000 + 7_000 * i, 900 + i, 0.45)
        fq = synth.reads_fastq(g, 200 + 40 * i, (100, 250), 0.005, 0.001, 60 + i)
        reqs.append((fq, i % 2 == 0))  # even: FASTQ bytes, odd: the parsed stream
    with Server(0, workers=2) as srv:
        futs = [srv.submit(fq if fx else synth.fastq_sequence_stream(fq), 31, 21, fastx=fx) for fq, fx in reqs]
        answers = [f.result(timeout=300) for f in futs]
    with T.Context(0) as ctx:
        for (fq, _), a in zip(reqs, answers):
            want = ctx.run(31, 21, fastx=fq)[0].sorted()
            got = T.Result(a.keys.copy(), a.counts.copy(), {}, 31).sorted()
            assert np.array_equal(got.keys, want.keys) and np.array_equal(got.counts, want.counts)


def test_served_batches_merge_and_match_the_oracle():
    """Requests queued while the workers are held (paused) are merged: a batch
    takes every waiting request of the oldest one's kind, so at least one batch
    holds several requests; every answer equals the oracle's count of that
    request alone (sorted pairs), for k = 21, 25, 31 interleaved."""
    import tuna_gb300 as T
    from oracle import oracle as O
    from tuna_gb300.serve import Server
    reqs = _requests()[:12]
    with Server(0, workers=2, paused=True) as srv:
        futs = [srv.submit(seq, k, m) for seq, k, m in reqs]
        srv.resume()
        answers = [f.result(timeout=300) for f in futs]
        sizes = list(srv.batch_sizes)
    assert max(sizes) >= 2 and sum(sizes) == len(reqs), sizes
    assert max(a.batch for a in answers) >= 2
    for (seq, k, m), a in zip(reqs, answers):
        want = O.count_stream(seq, k, m, threads=4)
        got = T.Result(np.asarray(a.keys).copy(), np.asarray(a.counts).copy(), {}, k).sorted()
        kw = (k + 31) // 32
        assert len(got) == len(want)
        assert np.array_equal(got.keys[:, :kw], want.keys) and np.array_equal(got.counts, want.counts)


def test_served_result_slabs_are_reused():
    """A worker's result memory is reused once the answers that view it are
    gone: many sequential requests allocate only a few slabs."""
    import gc
    from tuna_gb300.serve import Server
    reqs = _requests()[:3]
    with Server(0, workers=1) as srv:
        for _ in range(4):
            for seq, k, m in reqs:
                a = srv.submit(seq, k, m).result(timeout=300)
                assert len(a.keys) == len(a.counts)
                del a
                gc.collect()
        assert srv.batches == 12
