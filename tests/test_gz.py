"""gzip input (tg_read_input / tg_job_feed_file on ".gz" files): BGZF files
are cut at the member sizes in their 'BC' extra fields and inflated on several
host threads; any other gzip file is read as one stream, as the reference's
GzInput does (src/seq_source.hpp:48-141). Either way the bytes are the file's
inflated bytes, checked here against Python's gzip."""
import gzip
import os
import zlib

import numpy as np
import pytest

import tuna_gb300 as T

BGZF_EOF = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")


def bgzf(data: bytes, block: int = 65280, level: int = 6) -> bytes:
    """BGZF encoding: gzip members of at most `block` input bytes, each with
    the 'BC' extra subfield holding its total size minus one, then the empty
    end-of-file member."""
    out = bytearray()
    for i in range(0, len(data), block):
        chunk = data[i:i + block]
        c = zlib.compressobj(level, zlib.DEFLATED, -15)
        payload = c.compress(chunk) + c.flush()
        bsize = 18 + len(payload) + 8
        out += b"\x1f\x8b\x08\x04\x00\x00\x00\x00\x00\xff" + (6).to_bytes(2, "little")
        out += b"BC" + (2).to_bytes(2, "little") + (bsize - 1).to_bytes(2, "little")
        out += payload + zlib.crc32(chunk).to_bytes(4, "little") + len(chunk).to_bytes(4, "little")
    return bytes(out) + BGZF_EOF


def _fastq(seed: int, n: int = 3000) -> bytes:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.integers(50, 200))
        s = bytes(rng.choice(np.frombuffer(b"ACGTN", dtype=np.uint8), L, p=[.24, .25, .25, .25, .01]))
        out.append(b"@r%d\n" % i + s + b"\n+\n" + b"I" * L + b"\n")
    return b"".join(out)


def _write(tmp_path, name, data):
    p = os.path.join(tmp_path, name)
    with open(p, "wb") as f:
        f.write(data)
    return p


@pytest.mark.parametrize("threads", [1, 4, 16])
def test_bgzf_inflates_on_threads(tmp_path, threads):
    raw = _fastq(1, 6000)
    p = _write(tmp_path, "a.fq.gz", bgzf(raw, block=10_000))
    assert T.read_input(p, threads=threads) == raw


def test_other_gzip_read_as_one_stream(tmp_path):
    raw = _fastq(2)
    half = len(raw) // 2
    multi = gzip.compress(raw[:half]) + gzip.compress(raw[half:])  # two members, no size fields
    assert T.read_input(_write(tmp_path, "m.fq.gz", multi)) == raw
    assert T.read_input(_write(tmp_path, "s.fq.gz", gzip.compress(raw))) == raw


def test_plain_and_errors(tmp_path):
    raw = _fastq(3, 100)
    assert T.read_input(_write(tmp_path, "p.fq", raw)) == raw
    with pytest.raises(T.GpuError) as e:
        T.read_input(_write(tmp_path, "empty.fq", b""))
    assert "Empty file" in str(e.value)
    bad = bytearray(bgzf(raw, block=2000))
    bad[40] ^= 0xFF  # inside the first member's deflate data
    with pytest.raises(T.GpuError) as e:
        T.read_input(_write(tmp_path, "bad.fq.gz", bytes(bad)))
    assert "Cannot read" in str(e.value)
    with pytest.raises(T.GpuError):
        T.read_input(os.path.join(tmp_path, "missing.fq.gz"))


def test_bgzf_empty_members_only(tmp_path):
    with pytest.raises(T.GpuError) as e:
        T.read_input(_write(tmp_path, "eof.gz", BGZF_EOF))
    assert "Cannot read" in str(e.value)


@pytest.mark.gpu
def test_count_bgzf_file(tmp_path):
    from oracle import oracle as O
    raw = _fastq(4, 20_000)
    p = _write(tmp_path, "c.fq.gz", bgzf(raw))
    with T.Context(0) as ctx:
        got, _ = ctx.run(31, 21, files=[p])
    want = O.count_fastx(raw, 31, 21, threads=4)
    assert T.tsv_blob(got.keys, got.counts, 31) == O.tsv_blob(want)


def test_bgzf_claiming_more_than_memory_fails_cleanly(tmp_path):
    """Members whose sizes add up to ~800 TB: the reservation of the output
    fails on the host and comes back as a status with a message (no C++
    exception crosses the C ABI, the process goes on)."""
    member = (b"\x1f\x8b\x08\x04\x00\x00\x00\x00\x00\xff" + (6).to_bytes(2, "little") + b"BC"
              + (2).to_bytes(2, "little") + (27).to_bytes(2, "little") + b"\x03\x00"
              + (0).to_bytes(4, "little") + (0xFFFFFFFF).to_bytes(4, "little"))
    assert len(member) == 28
    p = _write(tmp_path, "huge.gz", member * 200_000)
    with pytest.raises(T.GpuError) as e:
        T.read_input(p, threads=4, cap=1 << 20)
    assert "host:" in str(e.value) or "Cannot read" in str(e.value)
    assert T.read_input(_write(tmp_path, "ok.gz", bgzf(b"ACGT\n"))) == b"ACGT\n"  # still usable


def test_inflated_far_beyond_the_first_guess(tmp_path):
    """A file that inflates to far more than the first buffer guess (64 x the
    compressed size) is read again at the size the library reports."""
    import gzip
    data = b">a\n" + b"A" * 20_000_000 + b"\n"
    p = _write(tmp_path, "big.fa.gz", gzip.compress(data, 9))
    assert os.path.getsize(p) * 64 < len(data)
    assert T.read_input(p) == data
    assert T.read_input(_write(tmp_path, "big_bgzf.fa.gz", bgzf(data)), threads=4) == data


def _member(chunk: bytes, pre_sub: bytes = b"") -> bytes:
    """One BGZF member whose extra field holds `pre_sub` before the BC subfield."""
    c = zlib.compressobj(6, zlib.DEFLATED, -15)
    payload = c.compress(chunk) + c.flush()
    xlen = len(pre_sub) + 6
    bsize = 12 + xlen + len(payload) + 8
    out = b"\x1f\x8b\x08\x04\x00\x00\x00\x00\x00\xff" + xlen.to_bytes(2, "little") + pre_sub
    out += b"BC" + (2).to_bytes(2, "little") + (bsize - 1).to_bytes(2, "little")
    return out + payload + zlib.crc32(chunk).to_bytes(4, "little") + len(chunk).to_bytes(4, "little")


def test_bgzf_edge_cases(tmp_path):
    """Other extra subfields before BC are skipped; a file that is not entirely
    BGZF members (truncated, or with bytes after the last member) is read as one
    gzip stream, as the reference's gzread loop reads every .gz file: a truncated
    file gives the bytes that inflate, trailing bytes are ignored. A member whose
    CRC does not match fails ("Cannot read"), where the reference's loop stops
    at the error and counts what it read before."""
    data = b">s\n" + b"ACGT" * 50000 + b"\n"
    chunks = [data[i:i + 30000] for i in range(0, len(data), 30000)]
    sub = b"RA" + (4).to_bytes(2, "little") + b"abcd"
    p = _write(tmp_path, "sub.gz", b"".join(_member(c, sub) for c in chunks) + BGZF_EOF)
    assert T.read_input(p, threads=4) == data
    full = bgzf(data, block=30000)
    got = T.read_input(_write(tmp_path, "trunc.gz", full[:-40]), threads=4)
    assert 0 < len(got) < len(data) and data.startswith(got)
    assert T.read_input(_write(tmp_path, "tail.gz", full + b"garbage!"), threads=4) == data
    bad = bytearray(full)
    bad[-len(BGZF_EOF) - 8] ^= 1  # the last data member's CRC
    with pytest.raises(T.GpuError) as e:
        T.read_input(_write(tmp_path, "crc.gz", bytes(bad)), threads=4)
    assert "Cannot read" in str(e.value)


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_large_plain_file_copied_out_on_threads(tmp_path, threads):
    """tg_read_input hands a 100 MB file back through its multi-threaded copy
    (shares of at least 16 MiB), byte for byte."""
    rng = np.random.default_rng(threads)
    data = b">s\n" + bytes(rng.choice(np.frombuffer(b"ACGTN\n", dtype=np.uint8), 100_000_000)) + b"\n"
    p = _write(tmp_path, "big.fa", data)
    assert T.read_input(p, threads=threads) == data
