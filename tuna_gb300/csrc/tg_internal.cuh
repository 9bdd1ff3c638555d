// tg_internal.cuh — shared definitions of the GB300 counting kernels.
//
// Data layout in HBM for one job (N = bytes of the sequence stream):
//   seq     u8[N]            ASCII stream; any byte outside [ACGTacgt] separates runs
//   packed  u32[]            2-bit kache codes (A0 C1 G2 T3), 16 bases per word,
//                            first base in bits 31:30 (MSB-first, like the
//                            reference's superkmer bytes); base g is stored at
//                            index g + TG_PAD, the TG_PAD leading bases are 0
//   valid   u32[]            1 bit per base, LSB-first, same TG_PAD offset
//   desc    u64[C][cap]      per Phase-1 CTA: one descriptor per superkmer record
//                            (start position, k-mer count, low 20 bits of its
//                            minimizer hash; see desc_pack)
//   binhist u32[2^20]        k-mer instances per bin (each sample owns a range of bins,
//                            one picked by minimizer hash); scanned into kofs
//   keys    u64 x W [K]      every canonical k-mer instance, grouped by bin
//                            (W = 1 for k <= 31)
//   out     keys + u32 counts of the distinct k-mers that pass ci/cx
//
// Reference counterparts (paths relative to the reference project root):
// kache codes src/partition_hash.hpp:68-70; the record byte layout the packed
// bases mirror src/superkmer_io.hpp:3-19; ntHash seeds and roll terms of
// HashTables include/nt_hash.hpp:26-124; the per-partition buckets the bins
// replace src/partition_hash.hpp:550-552; keys in the word layout of
// include/kache-hash/Kmer.hpp:38-48.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

constexpr int TG_PAD = 32;          // leading invalid bases in packed/valid
constexpr int CUT_TILE = 1024;      // k-mer start positions per tile of the export cut
constexpr int CUT_SPAN = 32768;     // the most positions any cut tile covers (array slack)
constexpr int CUT_THREADS = 256;
constexpr int MAX_W = 255;          // w = k - m
constexpr int P1_MAX = 4096;        // max segments of bins (gpu_parts), and partitions of the export cut
constexpr uint32_t NONE32 = 0xFFFFFFFFu;

// Event types of the Phase-1 tile event list.
constexpr uint32_t EV_OWNED = 1u;   // record start owned by this CTA
constexpr uint32_t EV_CUT = 2u;     // cut (record start of any owner or run end)

// ntHash tables for one m (include/nt_hash.hpp:26-40 seeds, :71-72 roll).
struct HashTables {
    // indexed by kache codes: FW[b] = FWD[nt(b)], RV[b] = REV[nt(b)]
    uint64_t FW[4], RV[4];
    uint64_t CTF[16], CTR[16];   // roll terms, index (out << 2) | in
    uint64_t GF[256], GR[256];   // 4-base group terms for initialisation
};

// Superkmer record descriptor (u64): the record covers the k-mers starting at
// positions [start, start + nk) of the stream; its bases are read from
// `packed` when it is counted. bin (20 bits) places the record's k-mers in the
// key array: the 2^20 bins are shared out among the samples of a job, sample s
// owning [base_s, base_s + 2^bits_s), and a record of sample s goes to bin
// base_s + (minimizer hash mod 2^bits_s). All instances of a canonical k-mer
// of one sample share its minimizer, hence its bin. (The export cut stores
// the low 20 bits of the minimizer hash there instead.)
constexpr int DESC_START_BITS = 36;
constexpr int BIN_BITS = 20;
__host__ __device__ __forceinline__ uint64_t desc_pack(uint64_t start, uint32_t nk, uint32_t bin) {
    return start | ((uint64_t)nk << DESC_START_BITS) | ((uint64_t)(bin & 0xFFFFFu) << 44);
}
__host__ __device__ __forceinline__ uint64_t desc_start(uint64_t d) { return d & ((1ull << DESC_START_BITS) - 1); }
__host__ __device__ __forceinline__ uint32_t desc_nk(uint64_t d) { return (uint32_t)(d >> DESC_START_BITS) & 0xFFu; }
__host__ __device__ __forceinline__ uint32_t desc_bin(uint64_t d) { return (uint32_t)(d >> 44); }

// Offset (in u32 units) of the u64 per-bucket k-mer counters that follow the
// u32 [P][C] record histogram: rounded up so the u64 array is 8-byte aligned
// whatever P * C is.
__host__ __device__ __forceinline__ uint64_t hist_kmers_offset(uint64_t p1, uint64_t n_cta) {
    return (p1 * n_cta + 1) & ~uint64_t(1);
}

struct CutParams {
    const uint32_t* packed;
    const uint32_t* valid;
    uint64_t n;              // sequence stream length (positions)
    int k, m, w;
    uint32_t L;              // max k-mers per record (forced split period)
    uint32_t p1_bits;        // log2 internal bucket count
    uint32_t n_cta;
    uint64_t chunk;          // k-mer start positions per CTA (multiple of CUT_TILE)
    uint64_t* desc;          // [n_cta][desc_cap] record descriptors
    uint64_t desc_cap;
    uint32_t* n_desc;        // [n_cta]
    uint32_t* hist;          // export cut: u32 [P][n_cta] records, then u64 [P] k-mers per bucket
    uint32_t* binhist;       // counting cut: [2^20] k-mers per bin
    // samples of the job (counting cut): sample i is positions [start[i], start[i+1])
    const unsigned long long* sample_start;  // [n_samples + 1]
    const uint32_t* sample_bin_base;         // [n_samples] first bin of each sample
    const uint8_t* sample_bin_bits;          // [n_samples] log2 bins of each sample
    uint32_t n_samples;
    unsigned long long* stats;  // [0] kmers, [1] records, [2] runs
    uint32_t* overflow;      // set when a CTA's descriptor list is full
    // export mode: full descriptors (start, minimizer hash, min_pos, nk)
    uint64_t* xdesc;         // [n_cta][desc_cap][3] or null
};

// Phase 2 works on slices of the phase-1 descriptor lists and on groups: runs
// of whole bins of one segment, whose keys are contiguous in the key array
// (the keys are laid out bin-major).
struct Slice {
    uint64_t r_lo, r_hi;  // descriptor range in the phase-1 lists
};

struct Group {
    unsigned long long lo, hi;  // key range [lo, hi)
    uint32_t parts, part;       // count only the keys whose hash part is `part` of `parts`
    uint32_t sample, pad;       // the sample whose keys these are
};

// A run of consecutive bins of one sample that k_plan cuts into groups.
struct Segment {
    uint32_t bin_lo, bin_hi, sample, pad;
};

// Counters of one Phase-2 run (device, u64 each).
enum P2Counter : int {
    P2C_NORMAL = 0,   // groups of at most `target` k-mers
    P2C_HEAVY,        // groups larger than `target`
    P2C_RETRY,        // groups pushed back for another pass with more parts
    P2C_FALLBACK,     // key ranges left to the global-memory table
    P2C_OUT,          // output cursor
    P2C_DISTINCT,     // distinct keys seen
    P2C_COUNT
};

struct KeysParams {
    const uint32_t* packed;
    const uint64_t* desc;              // phase-1 descriptor lists
    const Slice* slices;
    unsigned long long* kofs;          // [2^20 + 1] first key of each bin; a group's first bin's entry
                                       // is the group's cursor, advanced by k_keys
    uint32_t* gfirst;                  // [2^20] first bin of each bin's group (written by k_plan)
    const Segment* segs;               // k_plan: one warp per segment
    uint32_t n_segs;
    uint32_t target;                   // k-mer instances per group
    int k;
    void* keys;                        // u64 x W per k-mer instance
    Group* groups[2];                  // [0] normal, [1] heavy
    uint64_t groups_cap;
    unsigned long long* ctr;           // P2Counter
    uint32_t bin_lo, bin_hi;           // k_keys: only records of bins in [bin_lo, bin_hi)
};

struct CountParams {
    const void* keys;
    const Group* list[2];              // processed in order: list[1] first, then list[0]
    const unsigned long long* n_list;  // [0] entries of list[0], [1] of list[1]
    Group* retry;                      // failed groups, split in two
    unsigned long long* n_retry;
    uint64_t retry_cap;
    Group* fallback;
    uint64_t fallback_cap;
    uint64_t ci, cx;
    void* out_keys;                    // u64 x W per distinct k-mer
    uint32_t* out_counts;
    uint32_t* out_sample;              // sample of each pair (jobs of several samples), or null
    uint64_t out_cap;
    unsigned long long* ctr;           // P2Counter
    uint32_t smem_slots;               // table capacity in shared memory
    unsigned long long g_begin, g_end; // this launch counts groups [g_begin, g_end) of the sequence
    unsigned long long* work;          // this launch's group counter (starts at 0)
};

// A key range that did not fit in shared memory, counted in a global table.
struct FallbackParams {
    const void* keys;
    unsigned long long lo, hi;
    uint32_t parts, part, sample;
    void* tkeys;          // S slots
    uint32_t* tcnt;
    uint32_t mask;
    uint32_t* fail;
};

// Dynamic shared-memory cap of a kernel: the device's opt-in shared memory per
// block minus the kernel's static shared memory. It is a cap, not a
// reservation; every launch, from every host thread, sets this same value, so
// one thread's launch never finds the cap lowered by another's.
template <typename Kernel>
inline cudaError_t set_smem_cap(Kernel kernel, size_t need) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes a{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, kernel);
    if (e != cudaSuccess) return e;
    const size_t cap = (size_t)optin > a.sharedSizeBytes ? (size_t)optin - a.sharedSizeBytes : 0;
    if (need > cap) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap);
}

// ---------------------------------------------------------------- bit helpers
__device__ __forceinline__ uint64_t rol64(uint64_t x, int s) {
    s &= 63;
    return s ? (x << s) | (x >> (64 - s)) : x;
}
__device__ __forceinline__ uint64_t ror64(uint64_t x, int s) {
    s &= 63;
    return s ? (x >> s) | (x << (64 - s)) : x;
}

// 32 bases (64 bits, MSB-first) starting at array base index a.
__device__ __forceinline__ uint64_t window64(const uint32_t* pk, uint64_t a) {
    const uint64_t w = a >> 4;
    const uint32_t o = (uint32_t)(a & 15);
    const uint64_t hi = ((uint64_t)pk[w] << 32) | pk[w + 1];
    if (o == 0) return hi;
    return (hi << (2 * o)) | (pk[w + 2] >> (32 - 2 * o));
}

__device__ __forceinline__ uint32_t base_at(const uint32_t* pk, uint64_t a) {
    return (pk[a >> 4] >> (30 - 2 * (uint32_t)(a & 15))) & 3u;
}

// 64 validity bits starting at array base index a (bit 0 = base a).
__device__ __forceinline__ uint64_t valid64(const uint32_t* vb, uint64_t a) {
    const uint64_t w = a >> 5;
    const uint32_t o = (uint32_t)(a & 31);
    const uint64_t lo = ((uint64_t)vb[w + 1] << 32) | vb[w];
    if (o == 0) return lo;
    return (lo >> o) | ((uint64_t)vb[w + 2] << (64 - o));
}

__device__ __forceinline__ bool valid_base(const uint32_t* vb, uint64_t a) {
    return (vb[a >> 5] >> (a & 31)) & 1u;
}

// Canonical ntHash of the m-mer at array base index a, from scratch.
__device__ __forceinline__ void nt_init(const HashTables& T, const uint32_t* pk, uint64_t a, int m,
                                        uint64_t& fwd, uint64_t& rev) {
    const uint64_t win = window64(pk, a);
    uint64_t f = 0, r = 0;
    const int ng = m >> 2;
    for (int c = 0; c < ng; ++c) {
        const uint32_t v = (uint32_t)(win >> (56 - 8 * c)) & 0xFFu;
        f ^= rol64(T.GF[v], m - 4 - 4 * c);
        r ^= rol64(T.GR[v], 4 * c);
    }
    for (int i = 4 * ng; i < m; ++i) {
        const uint32_t b = (uint32_t)(win >> (62 - 2 * i)) & 3u;
        f ^= rol64(T.FW[b], m - 1 - i);
        r ^= rol64(T.RV[b], i);
    }
    fwd = f;
    rev = r;
}

__device__ __forceinline__ void nt_roll(const HashTables& T, uint32_t out, uint32_t in,
                                        uint64_t& fwd, uint64_t& rev) {
    const uint32_t idx = (out << 2) | in;
    fwd = rol64(fwd, 1) ^ T.CTF[idx];
    rev = ror64(rev, 1) ^ T.CTR[idx];
}

// ---------------------------------------------------------------- k-mer keys
// Reverse complement of a k-mer held in the low 2k bits (k <= 32).
__device__ __forceinline__ uint64_t revcomp64(uint64_t x, int k) {
    // complement = ~code; a full bit reversal reverses the 2-bit groups and
    // swaps the two bits inside each group, which the last step swaps back
    x = __brevll(~x);
    x = ((x >> 1) & 0x5555555555555555ull) | ((x & 0x5555555555555555ull) << 1);
    return x >> (64 - 2 * k);
}

struct K2 {
    uint64_t lo, hi;  // lo = last 32 bases, hi = the bases before them
};

__device__ __forceinline__ bool k2_less(const K2& a, const K2& b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// Reverse complement of a k-mer of 33..64 bases stored as (hi, lo).
__device__ __forceinline__ K2 revcomp128(const K2& x, int k) {
    // full 128-bit reversal of 2-bit groups, then shift right by 128 - 2k
    const uint64_t rlo = revcomp64(x.hi, 32);  // reversed hi becomes the low part
    const uint64_t rhi = revcomp64(x.lo, 32);
    const int sh = 128 - 2 * k;  // 2..64 for k in [32, 63]
    K2 r;
    if (sh >= 64) { r.lo = rhi >> (sh - 64); r.hi = 0; }
    else { r.lo = (rlo >> sh) | (rhi << (64 - sh)); r.hi = rhi >> sh; }
    return r;
}

__device__ __forceinline__ uint64_t mix_key1(uint64_t x) {
    x ^= x >> 31;
    x *= 0x9E3779B97F4A7C15ull;
    x ^= x >> 29;
    return x;
}
__device__ __forceinline__ uint64_t mix_key2(const K2& k) {
    return mix_key1(k.lo ^ mix_key1(k.hi + 0x632BE59BD9B4E019ull));
}

// ---------------------------------------------------------------- result digest
// Order-independent digest of (k-mer, count) pairs (tg_job_result_digest): two
// 64-bit terms per pair, summed mod 2^64. The words are the first nw =
// ceil(k/32) words of the key in the tuna::Kmer<k> layout (w1 is ignored when
// nw == 1); fa is MurmurHash3's 64-bit finaliser, fb SplitMix64's.
__host__ __device__ __forceinline__ uint64_t digest_fa(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}
__host__ __device__ __forceinline__ uint64_t digest_fb(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}
__host__ __device__ __forceinline__ void digest_terms(uint64_t w0, uint64_t w1, int nw, uint32_t count,
                                                      uint64_t& ta, uint64_t& tb) {
    uint64_t a = digest_fa(0x243F6A8885A308D3ull ^ w0), b = digest_fb(0x13198A2E03707344ull + w0);
    if (nw > 1) {
        a = digest_fa(a ^ w1);
        b = digest_fb(b + w1);
    }
    ta = digest_fa(a ^ ((uint64_t)count | (1ull << 40)));
    tb = digest_fb(b + ((uint64_t)count ^ 0xA4093822299F31D0ull));
}

}  // namespace tg
