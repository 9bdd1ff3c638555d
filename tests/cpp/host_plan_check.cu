// host_plan_check.cu — invariants of the host-side planning in libtuna_gpu.so
// (namespace tg), checked without a GPU: launch shapes and shared memory of
// the phase-1 cut for every (k, m) the GPU path accepts, buffer sizes, the
// record-descriptor packing, the output size bounds and the sharing of the
// 2^20 bins among the samples of a job.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "tg_launch.h"

using namespace tg;

static int fails = 0;
#define CHECK(cond, ...)                                           \
    do {                                                           \
        if (!(cond)) {                                             \
            if (++fails <= 20) {                                   \
                std::printf("FAIL line %d: ", __LINE__);           \
                std::printf(__VA_ARGS__);                          \
                std::printf("\n");                                 \
            }                                                      \
        }                                                          \
    } while (0)

static constexpr size_t SMEM_PER_CTA = 227u * 1024;  // opt-in shared memory of one CTA
static constexpr size_t SMEM_PER_SM = 228u * 1024;

static void check_cut_shapes() {
    for (int k = 2; k <= 63; ++k)
        for (int m = 1; m < k && m <= 32; ++m) {
            const int w = k - m;
            const size_t sm = cut_smem_bytes(w, k, 1, false);
            CHECK(sm <= SMEM_PER_CTA, "cut k=%d m=%d: %zu bytes of shared memory", k, m, sm);
            const uint32_t c = cut_ctas_per_sm(w, k, 1, false);
            CHECK(c >= 1 && (c == 1 || c * (sm + 1024) <= SMEM_PER_SM), "cut k=%d m=%d: %u CTAs of %zu bytes", k,
                  m, c, sm);
            CHECK(cut_tile(w, false) % 128 == 0, "cut k=%d m=%d: tile %llu", k, m,
                  (unsigned long long)cut_tile(w, false));
            const size_t se = cut_smem_bytes(w, k, 1, true);
            CHECK(se <= SMEM_PER_CTA, "export cut k=%d m=%d: %zu bytes", k, m, se);
            CHECK(cut_ctas_per_sm(w, k, 1, true) >= 1, "export cut k=%d m=%d: no CTA", k, m);
        }
}

static void check_buffers() {
    for (uint64_t n : {0ull, 1ull, 15ull, 16ull, 1000ull, 65536ull, 3100000024ull, (1ull << 36) - 1}) {
        const uint64_t pw = packed_words_for(n);
        CHECK(pw % 4 == 0, "packed words for %llu: %llu, not a multiple of 4", (unsigned long long)n,
              (unsigned long long)pw);
        // the cut reads up to a window and a span past the last base
        CHECK(pw * 16 >= TG_PAD + n + CUT_SPAN + 2 * (uint64_t)MAX_W, "packed words for %llu: %llu too few",
              (unsigned long long)n, (unsigned long long)pw);
    }
    for (int k = 2; k <= 63; ++k) {
        const int W = k <= 31 ? 1 : 2;
        // TSV: k letters, a tab, at most 10 digits of a u32 count, a line feed
        CHECK(fmt_max_bytes(TG_FMT_TSV, k, 1) >= (uint64_t)k + 12, "TSV bound k=%d", k);
        CHECK(fmt_max_bytes(TG_FMT_KFF, k, 3) == 3ull * ((k + 3) / 4 + 4), "KFF record size k=%d", k);
        CHECK(fmt_max_bytes(TG_FMT_RAW, k, 2) == 2ull * (8 * W + 4), "RAW record size k=%d", k);
        CHECK(key_bytes(W) == 8u * W, "key bytes W=%d", W);
    }
    CHECK(count_slots(1) > 0 && (count_slots(1) & (count_slots(1) - 1)) == 0, "table slots, 64-bit keys");
    CHECK(count_slots(2) > 0 && (count_slots(2) & (count_slots(2) - 1)) == 0, "table slots, 128-bit keys");
}

static void check_descriptors() {
    std::mt19937_64 rng(5);
    for (int i = 0; i < 100000; ++i) {
        const uint64_t start = i < 4 ? (i & 1 ? (1ull << DESC_START_BITS) - 1 : 0) : rng() & ((1ull << DESC_START_BITS) - 1);
        const uint32_t nk = i < 4 ? (i & 2 ? 255u : 1u) : (uint32_t)(rng() % 255 + 1);
        const uint32_t bin = i < 4 ? (i & 2 ? (1u << BIN_BITS) - 1 : 0u) : (uint32_t)(rng() & ((1u << BIN_BITS) - 1));
        const uint64_t d = desc_pack(start, nk, bin);
        CHECK(desc_start(d) == start && desc_nk(d) == nk && desc_bin(d) == bin, "descriptor %d round trip", i);
    }
}

// The bins of the samples: powers of two, contiguous and in order, inside the
// 2^20 bins, about in proportion to the samples' lengths; segments cover each
// sample's bins in order, none larger than seg_bins.
static void check_layout(const std::vector<unsigned long long>& starts, uint32_t seg_bins, const char* what) {
    const SampleBins B = layout_bins(starts, seg_bins);
    const size_t n = starts.size() - 1;
    CHECK(B.base.size() == n && B.bits.size() == n, "%s: %zu samples, %zu bases", what, n, B.base.size());
    if (B.base.size() != n) return;
    const double total = (double)std::max<unsigned long long>(1, starts[n] - starts[0]);
    const double all = (double)(1u << BIN_BITS);
    uint64_t next = 0;
    size_t sg = 0;
    for (size_t i = 0; i < n; ++i) {
        const uint64_t nb = 1ull << B.bits[i];
        CHECK(B.bits[i] <= BIN_BITS, "%s: sample %zu has %u bits", what, i, (unsigned)B.bits[i]);
        CHECK(B.base[i] == next, "%s: sample %zu starts at bin %u, not %llu", what, i, B.base[i],
              (unsigned long long)next);
        const double len = (double)(starts[i + 1] - starts[i]);
        const double share = all * len / total, low_share = (all - (double)n) * len / total;
        CHECK((double)nb <= std::max(1.0, share), "%s: sample %zu: %llu bins for a share of %.1f", what, i,
              (unsigned long long)nb, share);
        CHECK(B.bits[i] == BIN_BITS || (double)(2 * nb) > low_share, "%s: sample %zu: %llu bins, share %.1f", what,
              i, (unsigned long long)nb, low_share);
        uint64_t at = B.base[i];
        while (sg < B.segs.size() && B.segs[sg].sample == i) {
            const Segment& s = B.segs[sg];
            CHECK(s.bin_lo == at && s.bin_hi > s.bin_lo && s.bin_hi - s.bin_lo <= std::max<uint32_t>(1, seg_bins),
                  "%s: segment %zu [%u, %u) of sample %zu", what, sg, s.bin_lo, s.bin_hi, i);
            at = s.bin_hi;
            ++sg;
        }
        CHECK(at == B.base[i] + nb, "%s: sample %zu segments end at %llu, not %llu", what, i,
              (unsigned long long)at, (unsigned long long)(B.base[i] + nb));
        next += nb;
    }
    CHECK(sg == B.segs.size(), "%s: %zu segments left over", what, B.segs.size() - sg);
    CHECK(next <= (1ull << BIN_BITS), "%s: %llu bins used", what, (unsigned long long)next);
}

static std::vector<unsigned long long> starts_of(const std::vector<unsigned long long>& lens) {
    std::vector<unsigned long long> s{0};
    for (unsigned long long l : lens) s.push_back(s.back() + l + 1);  // one separator after each sample
    return s;
}

static void check_layouts() {
    std::mt19937_64 rng(11);
    std::vector<std::vector<unsigned long long>> cases;
    cases.push_back({3100000000ull});
    cases.push_back({1000, 1000});
    cases.push_back({0, 5, 0});
    std::vector<unsigned long long> v;
    for (int i = 0; i < 300; ++i) v.push_back(rng() % 2000000);
    cases.push_back(v);
    v.clear();
    for (int i = 0; i < 65536; ++i) v.push_back(rng() % 400);
    cases.push_back(v);
    v.assign(1000, 150);
    v.push_back(50000000000ull);
    cases.push_back(v);
    v.clear();
    for (int i = 0; i < 2000; ++i) v.push_back((unsigned long long)(1e4 * std::pow(5000.0, (double)(rng() % 10000) / 1e4)));
    cases.push_back(v);
    for (size_t c = 0; c < cases.size(); ++c)
        for (uint32_t seg_bits = 8; seg_bits <= 16; seg_bits += 4) {
            char what[64];
            std::snprintf(what, sizeof what, "case %zu, segments of 2^%u bins", c, seg_bits);
            check_layout(starts_of(cases[c]), 1u << seg_bits, what);
        }
}

int main() {
    check_cut_shapes();
    check_buffers();
    check_descriptors();
    check_layouts();
    if (fails) {
        std::printf("%d checks failed\n", fails);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
