#pragma once
// tuna/tuna.hpp — the reference's C++ counting API (include/tuna/tuna.hpp of the
// reference project) over the GB300 library libtuna_gpu.so.
//
// Same names, template parameters and error behaviour as the reference:
//
//   auto kmers = tuna::count_to<31>({"genome.fa"});           // unordered_map<string, uint32_t>
//   tuna::count<31>({"genome.fa"}, [](std::string_view kmer, uint32_t cnt) { ... });
//   tuna::count<31, 21>(files, [](const tuna::Kmer<31>& kmer, uint32_t cnt) { ... });
//   auto raw = tuna::count_to_raw<31>({"reads.fq.gz"});       // vector<pair<Kmer<31>, uint32_t>>
//
// Both phases run on the GPU; the callback is invoked from the calling thread
// only (the reference allows concurrent calls, so every reference callback is
// also correct here). Differences from the reference, by design of this path:
//   k is in [2, 63] (two 64-bit key words) and m in [1, min(k - 1, 32)];
//   Options::partitions only names the partition count (the GPU bins k-mers its
//   own way); Options::ram_gb is not used (the device budget is HBM);
//   Options::device selects the CUDA device.
//
// Build: g++ -std=c++17 -I<repo>/include app.cpp -L<dir of libtuna_gpu.so> -ltuna_gpu
//
// Reference behaviour mirrored (paths relative to the reference project root):
//   Options                      include/tuna/tuna.hpp:59-66
//   count<k, m, Callback>        include/tuna/tuna.hpp:91-151 (callback kind chosen
//                                at compile time as in src/count.hpp:288-293)
//   count_to<k, m, Container>    include/tuna/tuna.hpp:158-173
//   count_to_raw<k, m>           include/tuna/tuna.hpp:181-195
//   Kmer<k>::get_label           include/kache-hash/Kmer.hpp:664-682 (word 0 holds
//                                the last 32 bases, last base in the low bits)

#include <cstdint>
#include <cstring>
#include <filesystem>
#include <ostream>
#include <limits>
#include <mutex>
#include <stdexcept>
#include <string>
#include <string_view>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../tuna_gpu.h"

namespace tuna {

// Packed canonical k-mer: ceil(k/32) words, 2 bits per base (A0 C1 G2 T3),
// word 0 holds the last 32 bases with the last base in its two low bits (the
// layout of kache_hash::Kmer<k>, include/kache-hash/Kmer.hpp:38-48 of the
// reference). The members a counting callback uses are here with the
// reference's names and meaning: construction from a label, the labels
// (get_label, string_label, std::string conversion, operator<<), order and
// equality, base access (base_at, front, back; 2-bit codes where the reference
// returns DNA::Base, whose values are the same codes), data(), num_words(),
// as_int(), reverse_complement(), canonical(), write_packed_2bit_msb().
// Not provided: to_u64(seed) and Kmer_Hasher (they hash with the reference's
// vendored XXH3), the rolling and (k+1)-mer members (roll_*, from_prefix,
// from_suffix, from_super_kmer, lmer_at, in_forward), which only the reference's
// own counting loop uses.
template <uint16_t k>
struct Kmer {
    static_assert(k >= 2 && k <= 63, "tuna (GPU): k must be in [2, 63]");
    static constexpr uint16_t NUM_INTS = (k + 31) / 32;
    uint64_t kmer_data[NUM_INTS];

    Kmer() { std::memset(kmer_data, 0, sizeof kmer_data); }
    // From the k characters of label starting at label[kmer_idx] (ACGT, any case).
    Kmer(const char* label, std::size_t kmer_idx = 0) {
        std::memset(kmer_data, 0, sizeof kmer_data);
        for (uint16_t i = 0; i < k; ++i) {
            const char c = label[kmer_idx + i];
            const uint64_t b = (uint64_t)(((c >> 2) ^ (c >> 1)) & 3);  // A0 C1 G2 T3, case-folded
            const uint16_t from_end = (uint16_t)(k - 1 - i);
            kmer_data[from_end >> 5] |= b << (2 * (from_end & 31));
        }
    }
    explicit Kmer(const std::string& label, std::size_t kmer_idx = 0) : Kmer(label.c_str(), kmer_idx) {}

    static constexpr uint16_t num_words() { return NUM_INTS; }
    const uint64_t* data() const { return kmer_data; }
    uint64_t* data() { return kmer_data; }
    // The lowest word (the whole k-mer for k <= 32).
    uint64_t as_int() const { return kmer_data[0]; }

    // Base i of the k-mer (0 = first), as a 2-bit code.
    uint8_t base_at(uint16_t i) const {
        const uint16_t from_end = (uint16_t)(k - 1 - i);
        return (uint8_t)((kmer_data[from_end >> 5] >> (2 * (from_end & 31))) & 3u);
    }
    uint8_t front() const { return base_at(0); }
    uint8_t back() const { return base_at(k - 1); }

    Kmer reverse_complement() const {
        Kmer r;
        for (uint16_t i = 0; i < k; ++i) {
            const uint64_t b = 3u - base_at((uint16_t)(k - 1 - i));
            const uint16_t from_end = (uint16_t)(k - 1 - i);
            r.kmer_data[from_end >> 5] |= b << (2 * (from_end & 31));
        }
        return r;
    }
    // The smaller of the k-mer and its reverse complement (results of the
    // counting path are canonical already).
    Kmer canonical() const {
        const Kmer r = reverse_complement();
        return r < *this ? r : *this;
    }

    template <typename T_container_>
    void get_label(T_container_& label) const {
        label.resize(k);
        for (uint16_t i = 0; i < k; ++i) label[i] = "ACGT"[base_at(i)];
    }
    std::string string_label() const {
        std::string s;
        get_label(s);
        return s;
    }
    operator std::string() const { return string_label(); }
    // ceil(k/4) bytes, first base in the two high bits of byte 0 (the KFF
    // layout of the reference's write_packed_2bit_msb).
    void write_packed_2bit_msb(uint8_t* dst) const {
        std::memset(dst, 0, (k + 3) / 4);
        for (uint16_t i = 0; i < k; ++i) dst[i >> 2] |= (uint8_t)(base_at(i) << (6 - 2 * (i & 3)));
    }

    bool operator==(const Kmer& o) const { return std::memcmp(kmer_data, o.kmer_data, sizeof kmer_data) == 0; }
    bool operator!=(const Kmer& o) const { return !(*this == o); }
    // lexicographic order of the bases (A < C < G < T)
    bool operator<(const Kmer& o) const {
        for (int w = NUM_INTS - 1; w >= 0; --w)
            if (kmer_data[w] != o.kmer_data[w]) return kmer_data[w] < o.kmer_data[w];
        return false;
    }
    bool operator>(const Kmer& o) const { return o < *this; }
    friend std::ostream& operator<<(std::ostream& out, const Kmer& km) { return out << km.string_label(); }
};

struct Options {
    uint32_t threads = 1;                                         // host threads (parsing, formatting)
    uint32_t min_count = 1;                                       // only yield k-mers with count >= min_count
    uint32_t max_count = std::numeric_limits<uint32_t>::max();   // ... and <= max_count
    uint32_t partitions = 0;                                      // 0 = auto; rounded up to a power of two
    uint32_t ram_gb = 0;                                          // not used on the GPU path
    std::string work_dir;                                         // created if given; nothing is written there
    int device = 0;                                               // CUDA device
};

namespace detail {

inline uint32_t round_pow2(uint32_t v) {
    uint32_t p = 1;
    while (p < v && p < (1u << 31)) p <<= 1;
    return p;
}

// Status -> the reference's exception types.
[[noreturn]] inline void raise(tg_status s, const std::string& msg) {
    if (s == TG_ERR_ARG || s == TG_ERR_UNSUPPORTED) throw std::invalid_argument("tuna: " + msg);
    throw std::runtime_error("tuna: " + msg);
}

class Session {
public:
    explicit Session(const Options& o) {
        tg_ctx_opts co{};
        co.device = o.device;
        co.host_threads = o.threads;
        const tg_status s = tg_ctx_create(&co, &ctx_);
        if (s != TG_OK) raise(s, ctx_ ? tg_last_error(ctx_) : "no CUDA device for the counting library");
    }
    ~Session() {
        if (job_) tg_job_end(job_);
        if (ctx_) tg_ctx_destroy(ctx_);
    }
    Session(const Session&) = delete;
    Session& operator=(const Session&) = delete;
    void check(tg_status s) const {
        if (s != TG_OK) raise(s, tg_last_error(ctx_));
    }
    void begin(const tg_job_opts& jo) { check(tg_job_begin(ctx_, &jo, &job_)); }
    tg_job* job() const { return job_; }

private:
    tg_ctx* ctx_ = nullptr;
    tg_job* job_ = nullptr;
};

// Runs both phases over the files and hands the results to emit(words, counts,
// n, key_words) in chunks.
template <uint16_t k, uint16_t m, typename Emit>
void run(const std::vector<std::string>& files, const Options& opts, Emit&& emit) {
    static_assert(k >= 2 && k <= 63, "tuna (GPU): k must be in [2, 63]");
    static_assert(m >= 1 && m < k && m <= 32, "tuna (GPU): m must be in [1, min(k-1, 32)]");
    if (files.empty()) throw std::invalid_argument("tuna::count: no input files");
    if (!opts.work_dir.empty()) std::filesystem::create_directories(opts.work_dir);
    Session ss(opts);
    tg_job_opts jo{};
    jo.k = k;
    jo.m = m;
    jo.n_parts = opts.partitions ? round_pow2(opts.partitions) : 0;
    jo.ci = opts.min_count;
    jo.cx = opts.max_count;
    ss.begin(jo);
    for (const std::string& f : files) ss.check(tg_job_feed_file(ss.job(), f.c_str()));
    ss.check(tg_job_run(ss.job()));
    const uint64_t n = tg_job_result_size(ss.job());
    const int W = tg_job_key_words(ss.job());
    constexpr uint64_t CHUNK = 1u << 20;
    std::vector<uint64_t> words;
    std::vector<uint32_t> counts;
    for (uint64_t first = 0; first < n; first += CHUNK) {
        const uint64_t c = n - first < CHUNK ? n - first : CHUNK;
        words.resize(c * (uint64_t)W);
        counts.resize(c);
        ss.check(tg_job_result_copy(ss.job(), words.data(), counts.data(), first, c));
        emit(words.data(), counts.data(), c, W);
    }
}

}  // namespace detail

// Invokes cb(kmer, count) for each canonical k-mer that passes the count
// filters. ASCII callbacks take (std::string_view, uint32_t), binary ones
// (const tuna::Kmer<k>&, uint32_t); the kind is chosen at compile time.
// Throws std::invalid_argument if files is empty; std::runtime_error on a
// file, parse or device error.
template <uint16_t k, uint16_t m = 21, typename Callback>
void count(const std::vector<std::string>& files, Callback&& cb, Options opts = {}) {
    constexpr bool binary = std::is_invocable_v<Callback&, const Kmer<k>&, uint32_t>;
    detail::run<k, m>(files, opts, [&](const uint64_t* w, const uint32_t* c, uint64_t n, int W) {
        Kmer<k> km;
        std::string label;
        for (uint64_t i = 0; i < n; ++i) {
            std::memcpy(km.kmer_data, w + i * (uint64_t)W, sizeof km.kmer_data);
            if constexpr (binary) {
                cb(static_cast<const Kmer<k>&>(km), c[i]);
            } else {
                km.get_label(label);
                cb(std::string_view(label), c[i]);
            }
        }
    });
}

// Collects k-mer -> count pairs into Container (emplace(std::string, uint32_t)).
template <uint16_t k, uint16_t m = 21, typename Container = std::unordered_map<std::string, uint32_t>>
Container count_to(const std::vector<std::string>& files, Options opts = {}) {
    Container result;
    std::mutex mtx;
    count<k, m>(
        files,
        [&](std::string_view kmer, uint32_t cnt) {
            std::lock_guard<std::mutex> lg(mtx);
            result.emplace(std::string(kmer), cnt);
        },
        opts);
    return result;
}

// Binary variant of count_to: (Kmer<k>, count) pairs, no conversion to text.
template <uint16_t k, uint16_t m = 21>
std::vector<std::pair<Kmer<k>, uint32_t>> count_to_raw(const std::vector<std::string>& files, Options opts = {}) {
    std::vector<std::pair<Kmer<k>, uint32_t>> result;
    count<k, m>(files, [&](const Kmer<k>& kmer, uint32_t cnt) { result.emplace_back(kmer, cnt); }, opts);
    return result;
}

}  // namespace tuna
