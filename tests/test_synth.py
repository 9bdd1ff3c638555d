"""The seeded workload generators: well-formed output, fixed and variable read
lengths (the served workload's 100-250 bp reads), determinism."""
import numpy as np


def test_reads_variable_length_well_formed():
    from tuna_gb300 import synth
    g = synth.genome(40_000, 3, 0.45)
    fq = synth.reads_fastq(g, 5_000, (100, 250), 0.005, 0.001, 7)
    lines = fq.tobytes().split(b"\n")
    assert lines[-1] == b"" and (len(lines) - 1) % 4 == 0
    seqs, quals = lines[1::4], lines[3::4]
    assert len(seqs) == 5_000
    lens = np.array([len(s) for s in seqs])
    assert lens.min() >= 100 and lens.max() <= 250 and len(set(lens.tolist())) > 50
    assert all(len(q) == len(s) for s, q in zip(seqs, quals))
    assert all(h.startswith(b"@r") for h in lines[0::4][:-1])
    again = synth.reads_fastq(g, 5_000, (100, 250), 0.005, 0.001, 7)
    assert np.array_equal(fq, again)
    st = synth.fastq_sequence_stream(fq)
    assert st.size == int(lens.sum()) + 5_000


def test_reads_fixed_length():
    from tuna_gb300 import synth
    g = synth.genome(20_000, 4, 0.5)
    fq = synth.reads_fastq(g, 777, 150, 0.005, 0.0, 9)
    assert fq.size == 777 * (15 + 2 * 150 + 4)
