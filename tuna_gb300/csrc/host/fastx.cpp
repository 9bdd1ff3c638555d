// fastx.cpp — FASTA/FASTQ to sequence stream on the host.
//
// The reference parses with helicase (include/helicase_cpp/) configured to
// ignore headers and split at every non-ACGT byte (src/seq_source.hpp:33-39).
// The stream built here has the same runs: every ACGT run the reference hands
// to extract_superkmers_from_actg appears in the stream, in order, followed by
// a separator, and nothing else forms a run.
//
// FASTA (parser_fasta.hpp:233-316): bytes before the first '>' are ignored; a
// header runs from '>' to the next LF; in sequence, LF bytes are transparent
// (lines join) and every other non-ACGT byte ends the run. Since any non-ACGT
// byte in the stream is a separator, sequence lines are copied without their
// LF and each header becomes one separator.
//
// FASTQ (parser_fastq.hpp:112-285) is a 4-line record machine that walks the
// file in 64-byte blocks and keeps per block the mask of newlines not yet
// consumed. On malformed input (blank lines, a last line without LF) its result
// depends on that block walk, so the same walk is done here.
#include "tg_host.h"

#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>

namespace tgh {

static inline bool is_acgt(uint8_t x) {
    static const uint8_t lut[8] = {'A', 0, 'C', 0, 'T', 0, 'G', 0};
    return (uint8_t)(x & 0xDFu) == lut[x & 6u];
}

static void fasta_stream(const uint8_t* d, size_t n, std::vector<uint8_t>& out) {
    const uint8_t* p = static_cast<const uint8_t*>(memchr(d, '>', n));
    if (!p) return;
    const uint8_t* end = d + n;
    out.reserve(out.size() + n);
    while (p < end) {
        // p at '>': skip the header line including its LF
        const uint8_t* lf = static_cast<const uint8_t*>(memchr(p, '\n', (size_t)(end - p)));
        if (!lf) break;
        out.push_back('\n');
        p = lf + 1;
        // sequence lines until the next '>' (which may sit inside a line)
        while (p < end) {
            const uint8_t* nl = static_cast<const uint8_t*>(memchr(p, '\n', (size_t)(end - p)));
            const uint8_t* le = nl ? nl : end;
            const uint8_t* gt = static_cast<const uint8_t*>(memchr(p, '>', (size_t)(le - p)));
            if (gt) {
                out.insert(out.end(), p, gt);
                p = gt;
                break;
            }
            out.insert(out.end(), p, le);
            p = nl ? nl + 1 : end;
        }
    }
    out.push_back('\n');
}

namespace {
struct FqWalk {
    const uint8_t* d;
    size_t n;
    size_t blk = 0, blen = 0, pos = 0;
    uint64_t nl = 0, dna = 0;
    bool finished = false;
    int line = 0;

    void load(size_t b) {
        const size_t off = b * 64;
        blk = b;
        blen = (n - off) < 64 ? (n - off) : 64;
        pos = 0;
        uint64_t l = 0, a = 0;
        const uint8_t* q = d + off;
        if (blen == 64) {
            for (int i = 0; i < 64; ++i) {
                l |= (uint64_t)(q[i] == '\n') << i;
                a |= (uint64_t)is_acgt(q[i]) << i;
            }
        } else {
            for (size_t i = 0; i < blen; ++i) {
                l |= (uint64_t)(q[i] == '\n') << i;
                a |= (uint64_t)is_acgt(q[i]) << i;
            }
        }
        nl = l;
        dna = a & ~l;
    }
    bool advance() {  // true at end of input
        const size_t nb = blk + 1;
        if (nb * 64 >= n) { finished = true; return true; }
        load(nb);
        return false;
    }
    void incr() {
        if (pos + 1 < blen) ++pos;
        else advance();
    }
    void consume_nl() {
        nl &= nl - 1;
        incr();
        ++line;
    }
};
}  // namespace

static void fastq_stream(const uint8_t* d, size_t n, std::vector<uint8_t>& out) {
    FqWalk s{d, n};
    s.load(0);
    out.reserve(out.size() + n / 2 + 64);
    std::vector<uint8_t> run;
    for (;;) {
        switch (s.line & 3) {
        case 0:
            s.incr();
            if (s.finished) return;
            while (s.nl == 0)
                if (s.advance()) return;
            s.pos = (size_t)__builtin_ctzll(s.nl);
            s.consume_nl();
            break;
        case 1: {
            uint64_t mask = (s.dna | s.nl) & (~0ull << s.pos);
            while (mask == 0) {
                if (s.advance()) return;
                mask = s.dna | s.nl;
            }
            s.pos = (size_t)__builtin_ctzll(mask);
            if ((1ull << s.pos) & s.nl) { s.consume_nl(); continue; }
            run.clear();
            mask = ~s.dna & (~0ull << s.pos);
            size_t first = s.pos;
            while (mask == 0) {
                run.insert(run.end(), d + s.blk * 64 + s.pos, d + s.blk * 64 + s.blen);
                if (s.advance()) return;  // a run reaching the end of input is dropped
                first = 0;
                mask = ~s.dna;
            }
            s.pos = (size_t)__builtin_ctzll(mask);
            run.insert(run.end(), d + s.blk * 64 + first, d + s.blk * 64 + s.pos);
            if ((1ull << s.pos) & s.nl) s.consume_nl();
            out.insert(out.end(), run.begin(), run.end());
            out.push_back('\n');
            break;
        }
        case 2:
            while (s.nl == 0)
                if (s.advance()) return;
            s.pos = (size_t)__builtin_ctzll(s.nl);
            s.consume_nl();
            break;
        case 3:
            while (s.nl == 0)
                if (s.advance()) break;
            s.pos = s.nl ? (size_t)__builtin_ctzll(s.nl) : 64;
            s.consume_nl();
            break;
        }
    }
}

bool fastx_to_stream(const uint8_t* data, size_t len, std::vector<uint8_t>& out) {
    if (len == 0) return false;
    if (data[0] == '@') fastq_stream(data, len, out);
    else fasta_stream(data, len, out);
    return true;
}

// zlib is loaded at run time (libz.so.1), so the library builds without zlib
// development headers; gzip input fails with a clear message if it is absent.
namespace {
// z_stream as zlib.h lays it out (LP64), for the raw-deflate calls below
struct ZStream {
    const uint8_t* next_in;
    unsigned avail_in;
    unsigned long total_in;
    uint8_t* next_out;
    unsigned avail_out;
    unsigned long total_out;
    const char* msg;
    void* state;
    void* zalloc;
    void* zfree;
    void* opaque;
    int data_type;
    unsigned long adler;
    unsigned long reserved;
};
struct Zlib {
    using open_t = void* (*)(const char*, const char*);
    using read_t = int (*)(void*, void*, unsigned);
    using close_t = int (*)(void*);
    using buffer_t = int (*)(void*, unsigned);
    using init2_t = int (*)(ZStream*, int, const char*, int);
    using inflate_t = int (*)(ZStream*, int);
    using end_t = int (*)(ZStream*);
    using reset_t = int (*)(ZStream*);
    using crc_t = unsigned long (*)(unsigned long, const uint8_t*, unsigned);
    using version_t = const char* (*)();
    open_t gzopen = nullptr;
    read_t gzread = nullptr;
    close_t gzclose = nullptr;
    buffer_t gzbuffer = nullptr;
    init2_t inflateInit2_ = nullptr;
    inflate_t inflate = nullptr;
    end_t inflateEnd = nullptr;
    reset_t inflateReset = nullptr;
    crc_t crc32 = nullptr;
    version_t zlibVersion = nullptr;
    bool ok = false, raw_ok = false;
    Zlib() {
        void* h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) return;
        gzopen = reinterpret_cast<open_t>(dlsym(h, "gzopen"));
        gzread = reinterpret_cast<read_t>(dlsym(h, "gzread"));
        gzclose = reinterpret_cast<close_t>(dlsym(h, "gzclose"));
        gzbuffer = reinterpret_cast<buffer_t>(dlsym(h, "gzbuffer"));
        inflateInit2_ = reinterpret_cast<init2_t>(dlsym(h, "inflateInit2_"));
        inflate = reinterpret_cast<inflate_t>(dlsym(h, "inflate"));
        inflateEnd = reinterpret_cast<end_t>(dlsym(h, "inflateEnd"));
        inflateReset = reinterpret_cast<reset_t>(dlsym(h, "inflateReset"));
        crc32 = reinterpret_cast<crc_t>(dlsym(h, "crc32"));
        zlibVersion = reinterpret_cast<version_t>(dlsym(h, "zlibVersion"));
        ok = gzopen && gzread && gzclose;
        raw_ok = inflateInit2_ && inflate && inflateEnd && inflateReset && crc32 && zlibVersion;
    }
};
const Zlib& zlib() {
    static Zlib z;
    return z;
}

inline uint32_t le16(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
inline uint32_t le32(const uint8_t* p) { return le16(p) | (le16(p + 2) << 16); }

struct BgzfBlock {
    size_t cdata, clen;  // raw deflate payload in the file
    uint32_t isize, crc;
    size_t out;          // offset of its bytes in the inflated file
};

// BGZF (the blocked gzip of SAM/BAM and bgzip): every member carries its own
// size in the 'BC' extra subfield, so the members are found without
// inflating. False if the file is not entirely such members.
bool bgzf_blocks(const uint8_t* d, size_t n, std::vector<BgzfBlock>& out) {
    size_t off = 0, o = 0;
    while (off < n) {
        if (n - off < 26 || d[off] != 0x1F || d[off + 1] != 0x8B || d[off + 2] != 8 || d[off + 3] != 4) return false;
        const uint32_t xlen = le16(d + off + 10);
        if (n - off < 12 + (size_t)xlen + 8) return false;
        size_t bsize = 0;
        for (size_t x = off + 12; x + 4 <= off + 12 + xlen;) {
            const uint32_t slen = le16(d + x + 2);
            if (d[x] == 'B' && d[x + 1] == 'C' && slen == 2 && x + 6 <= off + 12 + xlen) bsize = le16(d + x + 4) + 1;
            x += 4 + slen;
        }
        if (bsize == 0 || bsize < 12 + (size_t)xlen + 8 || off + bsize > n) return false;
        BgzfBlock b;
        b.cdata = off + 12 + xlen;
        b.clen = bsize - (12 + xlen) - 8;
        b.crc = le32(d + off + bsize - 8);
        b.isize = le32(d + off + bsize - 4);
        b.out = o;
        o += b.isize;
        out.push_back(b);
        off += bsize;
    }
    return !out.empty();
}

// Inflates the blocks on `threads` host threads into out; false on a corrupt block.
bool bgzf_inflate(const Zlib& Z, const uint8_t* d, const std::vector<BgzfBlock>& blocks, unsigned threads,
                  Bytes& out) {
    const BgzfBlock& last = blocks.back();
    out.resize(last.out + last.isize);
    std::atomic<size_t> next{0};
    std::atomic<bool> bad{false};
    const size_t per = 64;  // blocks per claim (about 4 MiB of output)
    auto work = [&]() {
        ZStream zs{};
        if (Z.inflateInit2_(&zs, -15, Z.zlibVersion(), (int)sizeof(ZStream)) != 0) {
            bad = true;
            return;
        }
        for (;;) {
            const size_t b0 = next.fetch_add(per);
            if (b0 >= blocks.size() || bad) break;
            for (size_t i = b0; i < std::min(blocks.size(), b0 + per) && !bad; ++i) {
                const BgzfBlock& b = blocks[i];
                if (Z.inflateReset(&zs) != 0) { bad = true; break; }  // each block is its own raw stream
                zs.next_in = d + b.cdata;
                zs.avail_in = (unsigned)b.clen;
                zs.next_out = out.data() + b.out;
                zs.avail_out = b.isize;
                const unsigned long before = zs.total_out;
                const int r = Z.inflate(&zs, 4 /* Z_FINISH */);
                const bool ended = r == 1 /* Z_STREAM_END */ || (b.isize == 0 && b.crc == 0 && r == -5);
                if (!ended || zs.total_out - before != b.isize ||
                    Z.crc32(0, out.data() + b.out, b.isize) != b.crc)
                    bad = true;
            }
        }
        Z.inflateEnd(&zs);
    };
    threads = std::max(1u, std::min<unsigned>(threads, (unsigned)((blocks.size() + per - 1) / per)));
    std::vector<std::thread> th;
    th.reserve(threads);
    for (unsigned t = 1; t < threads; ++t) {
        try {
            th.emplace_back(work);
        } catch (...) {
            break;  // blocks are claimed from a shared counter: fewer threads take them all
        }
    }
    work();
    for (auto& t : th) t.join();
    return !bad;
}
}  // namespace

std::string read_input_file(const std::string& path, Bytes& out, unsigned threads) {
    const bool gz = path.size() > 3 && path.compare(path.size() - 3, 3, ".gz") == 0;
    if (gz) {
        const Zlib& Z = zlib();
        if (!Z.ok) return "gzip input needs libz.so.1: " + path;
        // BGZF: members found from their headers, inflated on all threads
        if (Z.raw_ok) {
            Bytes comp;
            FILE* f = fopen(path.c_str(), "rb");
            if (!f) return "Cannot open: " + path;
            fseek(f, 0, SEEK_END);
            const long sz = ftell(f);
            fseek(f, 0, SEEK_SET);
            if (sz > 0) {
                comp.resize((size_t)sz);
                const size_t r = fread(comp.data(), 1, comp.size(), f);
                if (r != comp.size()) comp.clear();
            }
            fclose(f);
            std::vector<BgzfBlock> blocks;
            if (!comp.empty() && bgzf_blocks(comp.data(), comp.size(), blocks)) {
                if (!bgzf_inflate(Z, comp.data(), blocks, threads, out)) return "Cannot read: " + path;
                if (out.empty()) return "Cannot read: " + path;
                return "";
            }
        }
        // any other gzip file: one stream through gzread, as the reference reads it
        void* f = Z.gzopen(path.c_str(), "rb");
        if (!f) return "Cannot open: " + path;
        if (Z.gzbuffer) Z.gzbuffer(f, 1u << 20);
        const size_t CH = 1u << 22;
        size_t got = 0;
        for (;;) {
            out.resize(got + CH);
            const int r = Z.gzread(f, out.data() + got, (unsigned)CH);
            if (r < 0) { Z.gzclose(f); out.resize(got); return "Cannot read: " + path; }
            got += (size_t)r;
            if (r == 0) break;
        }
        Z.gzclose(f);
        out.resize(got);
        if (got == 0) return "Cannot read: " + path;
        return "";
    }
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return "Cannot open file: " + path;
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (sz <= 0) { fclose(f); return "Empty file: " + path; }
    out.resize((size_t)sz);
    const size_t r = fread(out.data(), 1, (size_t)sz, f);
    fclose(f);
    if (r != (size_t)sz) return "Cannot read: " + path;
    return "";
}

}  // namespace tgh
