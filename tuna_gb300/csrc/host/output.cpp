// output.cpp — TSV / KFF / raw formatting of counted k-mers on the host.
//
// TSV: "<kmer>\t<count>\n", upper-case labels (src/count.hpp:180-216,
// Kmer::get_label Kmer.hpp:664-682). KFF: the container the reference fills
// through kff-cpp-api (src/kff_output.hpp:20-57): encoding A0 C1 G2 T3,
// unique and canonical flags, variables k, max = 1, data_size = 4, one raw
// section whose blocks hold one k-mer (ceil(k/4) bytes MSB-first,
// Kmer::write_packed_2bit_msb Kmer.hpp:685-693) and its count as 4 bytes
// big-endian.
#include "tg_host.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>

namespace tgh {

static inline void label_into(const uint64_t* w, int k, char* out) {
    static const char map[4] = {'A', 'C', 'G', 'T'};
    for (int i = 0; i < k; ++i) {
        const int b = k - 1 - i;
        out[i] = map[(w[b >> 5] >> (2 * (b & 31))) & 3];
    }
}

void format_tsv(const Pairs& p, uint64_t first, uint64_t n, std::string& out) {
    const size_t old = out.size();
    out.resize(old + n * (size_t)(p.k + 12));
    char* o = &out[old];
    for (uint64_t i = first; i < first + n; ++i) {
        label_into(p.keys + i * p.words, p.k, o);
        o += p.k;
        *o++ = '\t';
        char tmp[12];
        int t = 0;
        uint32_t c = p.counts[i];
        do { tmp[t++] = (char)('0' + c % 10); c /= 10; } while (c);
        while (t) *o++ = tmp[--t];
        *o++ = '\n';
    }
    out.resize((size_t)(o - out.data()));
}

void format_kff_entries(const Pairs& p, uint64_t first, uint64_t n, std::string& out) {
    const size_t kb = ((size_t)p.k + 3) / 4;
    const size_t old = out.size();
    out.resize(old + n * (kb + 4));
    uint8_t* o = reinterpret_cast<uint8_t*>(&out[old]);
    for (uint64_t i = first; i < first + n; ++i) {
        const uint64_t* w = p.keys + i * p.words;
        memset(o, 0, kb);
        for (int j = 0; j < p.k; ++j) {
            const int b = p.k - 1 - j;
            const unsigned c = (unsigned)((w[b >> 5] >> (2 * (b & 31))) & 3);
            o[j >> 2] |= (uint8_t)(c << (6 - 2 * (j & 3)));
        }
        o += kb;
        const uint32_t c = p.counts[i];
        o[0] = (uint8_t)(c >> 24); o[1] = (uint8_t)(c >> 16); o[2] = (uint8_t)(c >> 8); o[3] = (uint8_t)c;
        o += 4;
    }
}

void format_raw(const Pairs& p, uint64_t first, uint64_t n, std::string& out) {
    const size_t eb = 8 * (size_t)p.words + 4;
    const size_t old = out.size();
    out.resize(old + n * eb);
    char* o = &out[old];
    for (uint64_t i = first; i < first + n; ++i) {
        memcpy(o, p.keys + i * p.words, 8 * (size_t)p.words);
        memcpy(o + 8 * p.words, p.counts + i, 4);
        o += eb;
    }
}

static void put_be(std::string& s, uint64_t v, int n) {
    for (int i = n - 1; i >= 0; --i) s.push_back((char)((v >> (8 * i)) & 0xFF));
}
static void put_var(std::string& s, const char* name, uint64_t v) {
    s.append(name, strlen(name) + 1);
    put_be(s, v, 8);
}

std::string kff_header(int k, uint64_t n) {
    std::string s;
    s.append("KFF", 3);
    s.push_back(1);
    s.push_back(0);
    s.push_back((char)0x1B);  // A=00 C=01 G=10 T=11
    s.push_back(1);           // unique
    s.push_back(1);           // canonical
    put_be(s, 0, 4);          // no metadata
    s.push_back('v');
    put_be(s, 3, 8);
    put_var(s, "k", (uint64_t)k);
    put_var(s, "max", 1);
    put_var(s, "data_size", 4);
    s.push_back('r');
    put_be(s, n, 8);
    return s;
}

std::string kff_footer() {
    std::string s;
    const char* nm = "footer_size";
    const uint64_t fsz = 1 + 8 + strlen(nm) + 1 + 8 + 3;
    s.push_back('v');
    put_be(s, 1, 8);
    put_var(s, nm, fsz);
    s.append("KFF", 3);
    return s;
}

bool format_parallel(const Pairs& p, int fmt, unsigned threads,
                     bool (*sink)(const std::string& chunk, uint64_t npairs, void* user), void* user) {
    const uint64_t CH = 1u << 17;  // pairs per chunk
    const uint64_t nch = (p.n + CH - 1) / CH;
    if (nch == 0) return true;
    threads = std::max(1u, std::min<unsigned>(threads, (unsigned)std::min<uint64_t>(nch, 64)));
    // ring of formatted chunks, consumed in order by the calling thread
    const uint64_t RING = 2 * (uint64_t)threads;
    std::vector<std::string> buf(RING);
    std::vector<int> ready(RING, 0);
    std::mutex mu;
    std::condition_variable cv;
    std::atomic<uint64_t> next{0};
    uint64_t consumed = 0;
    bool stop = false;
    auto worker = [&]() {
        for (;;) {
            const uint64_t c = next.fetch_add(1);
            if (c >= nch) return;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || c < consumed + RING; });
                if (stop) return;
            }
            std::string s;
            const uint64_t f = c * CH, n = std::min(CH, p.n - f);
            if (fmt == 0) format_tsv(p, f, n, s);
            else if (fmt == 1) format_kff_entries(p, f, n, s);
            else format_raw(p, f, n, s);
            {
                std::lock_guard<std::mutex> lk(mu);
                buf[c % RING].swap(s);
                ready[c % RING] = 1;
            }
            cv.notify_all();
        }
    };
    std::vector<std::thread> th;
    for (unsigned i = 0; i < threads; ++i) th.emplace_back(worker);
    bool ok = true;
    for (uint64_t c = 0; c < nch; ++c) {
        std::string s;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return ready[c % RING] != 0; });
            s.swap(buf[c % RING]);
            ready[c % RING] = 0;
        }
        const uint64_t n = std::min(CH, p.n - c * CH);
        if (ok && !sink(s, n, user)) ok = false;
        {
            std::lock_guard<std::mutex> lk(mu);
            consumed = c + 1;
            if (!ok) stop = true;
        }
        cv.notify_all();
        if (!ok) break;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv.notify_all();
    for (auto& t : th) t.join();
    return ok;
}

}  // namespace tgh
