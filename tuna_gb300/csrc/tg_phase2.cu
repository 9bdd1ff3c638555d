// tg_phase2.cu — Phase 2 on the GPU: exact count of every canonical k-mer of
// every bucket record, ci/cx filter and compaction of the surviving pairs.
//
// Reference behaviour (paths relative to the reference project root):
//   every k-mer of a record       src/count.hpp:71-175 (the reference rolls through
//                                 the record's packed bases; here each k-mer is read
//                                 straight from the packed stream)
//   canonical form                include/kache-hash/Kmer.hpp:446-456, :629-646
//                                 (min of k-mer and reverse complement, word order)
//   count += 1 per instance       src/count.hpp:81, Streaming_Kmer_Hash_Table::upsert
//   keep ci <= count <= cx        src/count.hpp:202, :250, :287
//
// Pipeline (all instances of a canonical k-mer share its minimizer, hence its
// bin: the sample's first bin + minimizer hash bits; phase 1 counted the k-mer
// instances of every bin):
//   k_scan_*    bin counts -> key offsets
//   k_plan      per segment (a run of bins of one sample): groups of whole bins
//               of at most `target` k-mers
//   k_keys      every k-mer's canonical key, written at its group's cursor, so
//               the keys of a group are one contiguous range of the key array
//   k_count     persistent, one CTA per SM: each group's keys are read with
//               coalesced loads (the next round's already in flight while one
//               is counted) into a shared-memory open-addressing table, then
//               filtered and compacted.
//               A group with more distinct keys than the table holds comes back
//               as key-hash parts in the next launch (as many as its distinct
//               keys need, estimated); past MAX_PARTS parts it goes to the
//               global-memory table (k_fb_*).
#include <algorithm>
#include <vector>

#include "tg_launch.h"

namespace tg {

constexpr int P2_THREADS = 1024;         // threads of the phase-2 CTAs
constexpr int COUNT_THREADS = 1024;      // threads of a k_count CTA
constexpr int COUNT_PER_SM = 1;          // one CTA per SM: the largest table, the largest groups
constexpr uint32_t PROBE_LIMIT = 128;    // linear-probe steps before a group is split
constexpr uint32_t MAX_PARTS = 64;       // key-hash parts of one range before the global table
constexpr uint32_t SLICE_DESC = 65536;   // descriptors per slice
constexpr int KEYS_UNROLL = 4;           // k-mers per lane in flight in k_keys
constexpr uint64_t FALLBACK_CAP = 4096;

struct __align__(16) U128 {
    unsigned long long lo, hi;
};

template <int W>
struct KeyOps;

template <>
struct KeyOps<1> {
    using Key = unsigned long long;
    static constexpr size_t BYTES = 8;
    __device__ static Key empty() { return ~0ull; }
    __device__ static bool is_empty(const Key& k) { return k == ~0ull; }
    __device__ static bool eq(const Key& a, const Key& b) { return a == b; }
    __device__ static uint64_t hash(const Key& k) { return mix_key1(k); }
    __device__ static Key load(const Key* p) { return *reinterpret_cast<const volatile Key*>(p); }
    __device__ static Key cas(Key* p, const Key& cmp, const Key& val) { return atomicCAS(p, cmp, val); }
    __device__ static void store(void* out, uint64_t i, const Key& k) {
        reinterpret_cast<unsigned long long*>(out)[i] = k;
    }
};

template <>
struct KeyOps<2> {
    using Key = U128;
    static constexpr size_t BYTES = 16;
    __device__ static Key empty() { Key k; k.lo = ~0ull; k.hi = ~0ull; return k; }
    __device__ static bool is_empty(const Key& k) { return k.hi == ~0ull; }
    __device__ static bool eq(const Key& a, const Key& b) { return a.lo == b.lo && a.hi == b.hi; }
    __device__ static uint64_t hash(const Key& k) { K2 x{k.lo, k.hi}; return mix_key2(x); }
    __device__ static Key load(const Key* p) {
        const volatile unsigned long long* q = reinterpret_cast<const volatile unsigned long long*>(p);
        Key k; k.lo = q[0]; k.hi = q[1]; return k;
    }
    __device__ static Key cas(Key* p, const Key& cmp, const Key& val) { return atomicCAS(p, cmp, val); }
    __device__ static void store(void* out, uint64_t i, const Key& k) {
        reinterpret_cast<U128*>(out)[i] = k;
    }
};

// Key-hash part of a key (hash bits apart from the table's slot bits).
template <int W>
__device__ __forceinline__ uint32_t key_part(const typename KeyOps<W>::Key& key, uint32_t parts) {
    return (uint32_t)(KeyOps<W>::hash(key) >> 8) & (parts - 1);
}

// Insert one k-mer instance: count += 1. False if `limit` slots were taken.
// 64-bit keys are probed with a plain load and claimed with a CAS. A 128-bit
// key cannot be read in one single-copy-atomic load, and a read torn against a
// concurrent claim could skip the slot that holds the same k-mer, so 128-bit
// slots are probed with the CAS itself: it returns the whole current key.
template <int W>
__device__ __forceinline__ bool tbl_add(typename KeyOps<W>::Key* keys, uint32_t* cnt, uint32_t mask,
                                        const typename KeyOps<W>::Key& key, uint32_t limit) {
    using O = KeyOps<W>;
    uint32_t h = (uint32_t)(O::hash(key) >> 32) & mask;
    for (uint32_t p = 0; p < limit; ++p) {
        if constexpr (W == 1) {
            const typename O::Key cur = O::load(&keys[h]);
            if (O::eq(cur, key)) { atomicAdd(&cnt[h], 1u); return true; }
            if (O::is_empty(cur)) {
                const typename O::Key prev = O::cas(&keys[h], O::empty(), key);
                if (O::is_empty(prev) || O::eq(prev, key)) { atomicAdd(&cnt[h], 1u); return true; }
            }
        } else {
            const typename O::Key prev = O::cas(&keys[h], O::empty(), key);
            if (O::is_empty(prev) || O::eq(prev, key)) { atomicAdd(&cnt[h], 1u); return true; }
        }
        h = (h + 1) & mask;
    }
    return false;
}

// Canonical key of the k-mer starting at stream position s (bases read from
// the packed array; array index = s + TG_PAD).
template <int W>
__device__ __forceinline__ typename KeyOps<W>::Key kmer_key(const uint32_t* __restrict__ pk, uint64_t s, int k);

template <>
__device__ __forceinline__ unsigned long long kmer_key<1>(const uint32_t* __restrict__ pk, uint64_t s, int k) {
    const uint64_t a = s + TG_PAD;
    const uint64_t w = a >> 4;
    const uint32_t o = (uint32_t)(a & 15);
    const uint64_t hi = ((uint64_t)__ldg(pk + w) << 32) | __ldg(pk + w + 1);
    const uint64_t win = o ? (hi << (2 * o)) | (__ldg(pk + w + 2) >> (32 - 2 * o)) : hi;
    const uint64_t f = win >> (64 - 2 * k);
    const uint64_t r = revcomp64(f, k);
    return f < r ? f : r;
}

template <>
__device__ __forceinline__ U128 kmer_key<2>(const uint32_t* __restrict__ pk, uint64_t s, int k) {
    const uint64_t a = s + TG_PAD;
    const uint64_t w = a >> 4;
    const uint32_t o = (uint32_t)(a & 15);
    const uint32_t x0 = __ldg(pk + w), x1 = __ldg(pk + w + 1), x2 = __ldg(pk + w + 2), x3 = __ldg(pk + w + 3),
                   x4 = __ldg(pk + w + 4);
    uint64_t w01 = ((uint64_t)x0 << 32) | x1, w23 = ((uint64_t)x2 << 32) | x3;
    if (o) {
        w01 = (w01 << (2 * o)) | (x2 >> (32 - 2 * o));
        w23 = (w23 << (2 * o)) | (x4 >> (32 - 2 * o));
    }
    const int sh = 128 - 2 * k;  // 2..64
    K2 f;
    if (sh >= 64) { f.lo = w01 >> (sh - 64); f.hi = 0; }
    else { f.lo = (w23 >> sh) | (w01 << (64 - sh)); f.hi = w01 >> sh; }
    const K2 r = revcomp128(f, k);
    const K2& c = k2_less(f, r) ? f : r;
    U128 key;
    key.lo = c.lo;
    key.hi = c.hi;
    return key;
}

// ---------------------------------------------------------------- k_plan
// One warp per segment (a run of consecutive bins of one sample): its groups,
// from the scanned key offsets ko[bin]. Greedy, in bin order: a group starting
// at bin s takes the most bins e - s with at most `target` keys (one bin if that
// bin alone is larger; such a group is listed as heavy). Each step is one
// upper-bound search over ko, done by the warp as a 32-way search. Every bin of
// the group gets the group's first bin in gfirst: k_keys appends all of the
// group's keys at that bin's cursor.
constexpr int PLAN_THREADS = 256;

__global__ void __launch_bounds__(PLAN_THREADS) k_plan(KeysParams P) {
    const int lane = threadIdx.x & 31;
    const uint32_t sg = blockIdx.x * (PLAN_THREADS / 32) + (threadIdx.x >> 5);
    if (sg >= P.n_segs) return;  // warp-uniform
    const Segment seg = P.segs[sg];
    const uint32_t nb = seg.bin_hi - seg.bin_lo;
    const unsigned long long* ko = P.kofs + seg.bin_lo;
    const unsigned long long end = ko[nb];
    const unsigned long long T = P.target;
    uint32_t s = 0;
    unsigned long long ks = ko[0];
    while (ks < end) {
        // largest e in [s + 1, nb] with ko[e] <= ks + T (e = s + 1 if there is none)
        const unsigned long long lim = ks + T;
        uint32_t lo = s + 1, hi = nb;
        if (ko[lo] <= lim) {
            while (lo < hi) {  // invariant: ko[lo] <= lim, the answer is in [lo, hi]
                const uint32_t step = (hi - lo + 31) / 32;
                const uint32_t e = lo + (uint32_t)lane * step;
                const unsigned ok = __ballot_sync(0xffffffffu, e <= hi && ko[e] <= lim);  // bit 0 is set
                const int l = 31 - __clz(ok);
                const uint32_t nlo = lo + (uint32_t)l * step;
                hi = l == 31 ? hi : min(nlo + step - 1, hi);
                lo = nlo;
            }
        }
        const uint32_t e = lo;
        const unsigned long long ke = ko[e];
        for (uint32_t b = s + (uint32_t)lane; b < e; b += 32) P.gfirst[seg.bin_lo + b] = seg.bin_lo + s;
        if (lane == 0) {
            const int heavy = ke - ks > T ? 1 : 0;
            const unsigned long long q = atomicAdd(&P.ctr[heavy ? P2C_HEAVY : P2C_NORMAL], 1ull);
            if (q < P.groups_cap) {
                Group g;
                g.lo = ks;
                g.hi = ke;
                g.parts = 1;
                g.part = 0;
                g.sample = seg.sample;
                g.pad = 0;
                P.groups[heavy][q] = g;
            }
        }
        s = e;
        ks = ke;
    }
}

// ---------------------------------------------------------------- k_keys
// Every k-mer of a slice of the phase-1 descriptor lists (in stream order, so
// the packed bases are read front to back): canonical key written at its
// group's cursor (the cursor of the group's first bin, gfirst). A warp takes 32
// descriptors at a time; each reserves its k-mers' places with one global
// atomic on that cursor, then the warp's lanes take the batch's k-mers in order
// (consecutive lanes, consecutive keys). Keys appended per group rather than
// per bin: a group's keys are the same contiguous range, in another order
// inside it, with about a third as many places being written at once (groups
// of ~3 bins), so more of the partly written sectors are completed in L2.
// The descriptors are loaded two batches ahead and the next batch's gfirst
// entries one batch ahead, and each batch's atomic is issued before the
// previous batch's keys are made (k_keys 19.8 -> 19.1 ms at 3.1 G keys).
//
// A run restricted to a range of bins (the passes of a job larger than the
// memory budget) keeps only the records of those bins, moved to the front of
// the warp's batch so that every active lane still holds one record.
template <int W>
__global__ void __launch_bounds__(P2_THREADS) k_keys(KeysParams P) {
    using O = KeyOps<W>;
    __shared__ uint64_t s_keep[P2_THREADS];
    __shared__ uint32_t s_keepg[P2_THREADS];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const Slice sl = P.slices[blockIdx.x];
    const uint64_t* d = P.desc + sl.r_lo;
    const uint32_t n = (uint32_t)(sl.r_hi - sl.r_lo);
    const int k = P.k;
    const bool filt = P.bin_lo != 0 || P.bin_hi != (1u << BIN_BITS);
    auto load_desc = [&](uint32_t i) -> uint64_t { return i < n ? d[i] : 0; };
    // gfirst of a descriptor's bin (any bin of a descriptor is below 2^20;
    // bins outside this run's range are read but not used)
    auto group_of = [&](uint64_t dv) -> uint32_t { return desc_nk(dv) ? P.gfirst[desc_bin(dv)] : 0u; };
    const uint32_t b0 = (uint32_t)wid * 32 + lane;
    uint64_t dnext = load_desc(b0);                 // batch i + 1 (loaded)
    uint32_t gnext = group_of(dnext);
    uint64_t dnext2 = load_desc(b0 + P2_THREADS);   // batch i + 2 (in flight)
    // A batch is prepared (restricted to this run's bins, moved to the front of
    // the warp; its places reserved by the atomic) one batch ahead: the atomic's
    // round trip overlaps the previous batch's keys.
    auto prepare = [&](uint64_t& dv, uint32_t gv, unsigned long long& koff) {
        koff = 0;
        if (filt) {
            const uint32_t b = desc_bin(dv);
            const bool keep = desc_nk(dv) && b >= P.bin_lo && b < P.bin_hi;
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const uint32_t j = wid * 32 + __popc(m & ((1u << lane) - 1u));
                s_keep[j] = dv;
                s_keepg[j] = gv;
            }
            __syncwarp();
            dv = lane < __popc(m) ? s_keep[wid * 32 + lane] : 0;
            gv = lane < __popc(m) ? s_keepg[wid * 32 + lane] : 0;
            __syncwarp();
        }
        const uint32_t nk = desc_nk(dv);  // 0 past the slice; at least 1 otherwise
        if (nk) koff = atomicAdd(&P.kofs[gv], (unsigned long long)nk);
    };
    uint64_t cdv = dnext;
    unsigned long long ckoff;
    {
        const uint32_t cg = gnext;
        dnext = dnext2;
        gnext = group_of(dnext);
        dnext2 = load_desc(b0 + 2 * P2_THREADS);
        prepare(cdv, cg, ckoff);
    }
    for (uint32_t base = (uint32_t)wid * 32; base < n; base += P2_THREADS) {
        uint64_t ndv = dnext;
        unsigned long long nkoff;
        {
            const uint32_t ng = gnext;
            dnext = dnext2;
            gnext = group_of(dnext);
            dnext2 = load_desc(base + 3 * P2_THREADS + lane);
            prepare(ndv, ng, nkoff);
        }
        const uint64_t dv = cdv;
        const unsigned long long koff = ckoff;
        cdv = ndv;
        ckoff = nkoff;
        const uint32_t nk = desc_nk(dv);
        uint32_t incl = nk;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t excl = incl - nk;
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        // k-mer t of the batch belongs to lane o: stream position srcb_o + t,
        // key index dstb_o + t
        const uint64_t srcb = desc_start(dv) - excl;
        const uint64_t dstb = koff - excl;
        for (uint32_t t0 = 0; t0 < total; t0 += 32 * KEYS_UNROLL) {
            typename O::Key kv[KEYS_UNROLL];
            uint64_t dst[KEYS_UNROLL];
            bool act[KEYS_UNROLL];
#pragma unroll
            for (int u = 0; u < KEYS_UNROLL; ++u) {
                const uint32_t r0 = t0 + 32 * u;  // warp-uniform
                act[u] = false;
                if (r0 >= total) continue;
                // owner of k-mer r0 + l = (lanes starting before r0) + (starts in
                // [r0, r0 + l]) - 1; starts are distinct since every nk >= 1
                const uint32_t rel = excl - r0;
                const unsigned starts = __reduce_or_sync(0xffffffffu, (nk && rel < 32) ? 1u << rel : 0u);
                const unsigned before = __popc(__ballot_sync(0xffffffffu, excl < r0));
                const uint32_t own = (before + __popc(starts & ((2u << lane) - 1u)) - 1u) & 31u;
                const uint64_t sb = __shfl_sync(0xffffffffu, srcb, own);
                const uint64_t db = __shfl_sync(0xffffffffu, dstb, own);
                const uint32_t t = r0 + lane;
                act[u] = t < total;
                if (act[u]) {
                    kv[u] = kmer_key<W>(P.packed, sb + t, k);
                    dst[u] = db + t;
                }
            }
#pragma unroll
            for (int u = 0; u < KEYS_UNROLL; ++u)
                if (act[u]) O::store(P.keys, dst[u], kv[u]);
        }
    }
}

// ---------------------------------------------------------------- k_count
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// A slot's count in shared memory is its key's occurrences after the first:
// the thread that claims a slot adds nothing (its key counts through the claim),
// later occurrences add 1, and the output count is the stored value + 1. Most
// keys of a group occur once, so most keys take one shared atomic (the CAS),
// not two.
//
// 128-bit keys: slots probed in order from the home slot h with the CAS itself
// (a 128-bit key cannot be read in one single-copy-atomic load, and a torn
// read could skip the slot that holds the same k-mer). Returns 1 for a new key,
// 0 for a known one, -1 after PROBE_LIMIT slots.
__device__ __forceinline__ int claim_cas(U128* keys, uint32_t* cnt, uint32_t mask, const U128& key, uint32_t h,
                                         uint32_t& slot) {
    using O = KeyOps<2>;
    for (uint32_t p = 0; p < PROBE_LIMIT; ++p) {
        const U128 prev = O::cas(&keys[h], O::empty(), key);
        if (O::is_empty(prev)) { slot = h; return 1; }
        if (O::eq(prev, key)) { atomicAdd(&cnt[h], 1u); return 0; }
        h = (h + 1) & mask;
    }
    return -1;
}

// The 64-bit table as buckets of 4 slots (32 bytes). A key's probe order is
// fixed: its home slot, then the slots of its home bucket (which holds the home
// slot) in order, then the next bucket's, and so on; a key takes the first slot
// of that order that is empty when it comes, and slots are never emptied during
// a group, so two inserts of one key meet in the same slot. After the home slot
// one probe reads a whole bucket (two 16-byte loads; each 8-byte slot is read
// atomically). If the key
// is in the bucket, it is counted there (a slot once taken keeps its key);
// otherwise the first empty slot is claimed by CAS, and a CAS lost to another
// key re-reads the bucket. Returns 1 for a new key, 0 for a known one, -1 after
// PROBE_BUCKETS buckets.
constexpr uint32_t BUCKET = 4;
constexpr uint32_t PROBE_BUCKETS = 32;

__device__ __forceinline__ void lds_bucket(const unsigned long long* p, unsigned long long (&v)[BUCKET]) {
    const uint32_t a = smem_addr(p);
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2];" : "=l"(v[0]), "=l"(v[1]) : "r"(a));
    asm volatile("ld.volatile.shared.v2.u64 {%0, %1}, [%2+16];" : "=l"(v[2]), "=l"(v[3]) : "r"(a));
}

__device__ __forceinline__ int claim_bucket(unsigned long long* keys, uint32_t* cnt, uint32_t bmask,
                                            unsigned long long key, uint32_t hs, uint32_t& slot) {
    // the home slot first (one 8-byte load): in a table at most half full it is
    // usually empty or holds the key (20 % less k_count time than reading the
    // whole bucket first); the probe order goes on with the home bucket's slots
    {
        unsigned long long v0;
        asm volatile("ld.volatile.shared.u64 %0, [%1];" : "=l"(v0) : "r"(smem_addr(keys + hs)));
        if (v0 == key) { atomicAdd(&cnt[hs], 1u); return 0; }
        if (v0 == ~0ull) {
            const unsigned long long prev = atomicCAS(&keys[hs], ~0ull, key);
            if (prev == ~0ull) { slot = hs; return 1; }
            if (prev == key) { atomicAdd(&cnt[hs], 1u); return 0; }
        }
    }
    uint32_t b = hs / BUCKET;
    for (uint32_t p = 0; p < PROBE_BUCKETS;) {
        unsigned long long v[BUCKET];
        lds_bucket(keys + b * BUCKET, v);
        int hit = -1, emp = -1;
#pragma unroll
        for (int j = BUCKET - 1; j >= 0; --j) {
            if (v[j] == key) hit = j;
            if (v[j] == ~0ull) emp = j;
        }
        if (hit >= 0) { atomicAdd(&cnt[b * BUCKET + hit], 1u); return 0; }
        if (emp < 0) { b = (b + 1) & bmask; ++p; continue; }
        const unsigned long long prev = atomicCAS(&keys[b * BUCKET + emp], ~0ull, key);
        if (prev == ~0ull) { slot = b * BUCKET + emp; return 1; }
        if (prev == key) { atomicAdd(&cnt[b * BUCKET + emp], 1u); return 0; }
        // the slot went to another key: read the bucket again
    }
    return -1;
}

// Asynchronous copy (cp.async, two 16-byte pieces) of group `gi` of the
// launch's sequence (list 1 first, then list 0) into shared memory; an index
// past the end gives an empty group.
__device__ __forceinline__ void copy_group(Group* dst, const CountParams& P, unsigned long long gi,
                                           unsigned long long n1, unsigned long long ntot) {
    if (gi >= ntot) {
        dst->lo = dst->hi = 0;
        dst->parts = 0;
        return;
    }
    const Group* src = gi < n1 ? P.list[1] + gi : P.list[0] + (gi - n1);
    const uint32_t d = smem_addr(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d + 16),
                 "l"(reinterpret_cast<const uint8_t*>(src) + 16)
                 : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int W>
struct CountSmem {
    size_t keys, cnt, list, total;
    __host__ __device__ void layout(uint32_t slots) {
        size_t o = 0;
        keys = o; o += KeyOps<W>::BYTES * (size_t)slots;
        cnt = o; o += 4 * (size_t)slots;
        list = o; o += 2 * (size_t)slots;  // slots claimed by the group, in claim order
        total = (o + 15) & ~size_t(15);
    }
};

// Persistent: COUNT_PER_SM CTAs per SM take groups in order (list 1, then list 0) from a
// global counter. A group's keys are one contiguous range; they are inserted
// in rounds of RK keys, thread t taking keys t, t + COUNT_THREADS, ... of a round,
// and each thread's keys of the next round (or of the next group's first round)
// are loaded into registers while it inserts the current ones, so there is no
// barrier inside a group. Every slot a key claims goes onto a list in shared
// memory (each round's new slots placed with one shared atomic per warp), so
// after the group the threads walk the list, not the table: pair i of the group
// is written to out[base + i] (coalesced) and its slot cleared. With ci/cx
// limits the table is scanned instead and the kept pairs compacted by ballots.
// A group with more distinct keys than 7/8 of the table (or a probe run past
// the limit) comes back as F key-hash parts, F the power of two that gives
// half-full tables for its distinct keys: known when the group ran to its end,
// else estimated from the keys seen before the table filled. Halving at every
// level instead re-read a heavy bin's keys once per level (all of k_count at
// 3.1 G keys: 47.4 -> 41.9 ms). Group entries are fetched
// two groups ahead (cp.async) into a ring of three. Groups are planned at half
// the table (`target`): with the list the table's size no longer costs a scan,
// and a half-full table has fewer collisions (measured: 0.7 -> 0.5 of the
// table, 16.1 -> 14.0 ms for 0.93 G keys).
template <int W>
//
// At most 56 registers per thread (no spills; 64 without the cap): 1,024 x 56
// leaves 8,192 of the SM's registers, room for one CTA of the host-link copy
// (tg_link.cu: 256 threads x 32 registers) beside each counting CTA, so the
// copy of a wave's pairs to host memory runs while the next wave counts.
__global__ void __maxnreg__(56) k_count(CountParams P) {
    using O = KeyOps<W>;
    using Key = typename O::Key;
    constexpr int U = W == 1 ? 4 : 2;                 // keys per thread per round
    constexpr uint32_t RK = U * COUNT_THREADS;           // keys per round
    constexpr uint32_t SPT = W == 1 ? 16 : 8;         // table slots per thread
    extern __shared__ __align__(128) uint8_t smem[];
    CountSmem<W> L;
    L.layout(P.smem_slots);
    Key* keys = reinterpret_cast<Key*>(smem + L.keys);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + L.cnt);
    uint16_t* list = reinterpret_cast<uint16_t*>(smem + L.list);
    __shared__ uint32_t s_nlist;                      // entries of list
    __shared__ __align__(16) Group s_grp[3];          // groups g, g + 1, g + 2
    __shared__ uint32_t s_fail;
    __shared__ uint32_t s_bad;  // round in which a probe first gave up (the table was full); ~0: none
    __shared__ uint32_t s_wnew[COUNT_THREADS / 32];      // new keys of the group, per warp
    __shared__ uint32_t s_wout[COUNT_THREADS / 32];      // output keys per warp, then their offsets
    __shared__ unsigned long long s_obase;

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t S = P.smem_slots, mask = S - 1;    // S == SPT * COUNT_THREADS
    const uint32_t fill_cap = S - S / 8;
    // counts are at least 1 and fit in 32 bits: without ci/cx limits every key is kept
    const bool filtered = P.ci > 1 || P.cx < 0xFFFFFFFFull;
    const unsigned long long n1 = P.n_list[1];
    const unsigned long long ntot = min(P.n_list[0] + n1, P.g_end);
    const unsigned long long g0 = P.g_begin;
    const Key* src = static_cast<const Key*>(P.keys);
    unsigned long long distinct = 0;                  // per warp, in lane 0

    for (uint32_t i = tid; i < S; i += COUNT_THREADS) { keys[i] = O::empty(); cnt[i] = 0; }
    if (tid < COUNT_THREADS / 32) s_wnew[tid] = 0;
    unsigned long long gi_pend = ~0ull;               // thread 0: index of group g + 3
    if (tid == 0) {
        s_fail = 0;
        s_bad = ~0u;
        s_nlist = 0;
        for (int q = 0; q < 3; ++q) copy_group(&s_grp[q], P, g0 + atomicAdd(P.work, 1ull), n1, ntot);
        gi_pend = g0 + atomicAdd(P.work, 1ull);
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    __syncthreads();

    // keys of round r of group g into K (EMPTY past the group's end)
    auto load_round = [&](const Group& g, uint32_t r, Key (&K)[U]) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned long long i = g.lo + (unsigned long long)r * RK + (uint32_t)u * COUNT_THREADS + tid;
            K[u] = i < g.hi ? src[i] : O::empty();
        }
    };

    Key K[U];
    {
        const Group g0 = s_grp[0];
        load_round(g0, 0, K);
    }
    for (uint32_t q = 0;; q = q == 2 ? 0 : q + 1) {
        const Group g = s_grp[q];
        if (g.hi <= g.lo) break;  // no more groups
        const uint32_t nr = (uint32_t)((g.hi - g.lo + RK - 1) / RK);
        bool bad = false;
        for (uint32_t r = 0; r < nr; ++r) {
            Key N[U];
            if (r + 1 < nr) load_round(g, r + 1, N);
            else load_round(s_grp[q == 2 ? 0 : q + 1], 0, N);
            uint32_t newm = 0, nsl[U];
            if (!bad) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    nsl[u] = 0;
                    if (bad || O::is_empty(K[u])) continue;
                    const uint64_t h = O::hash(K[u]);
                    if (g.parts > 1 && ((uint32_t)(h >> 8) & (g.parts - 1)) != g.part) continue;
                    int res;
                    if constexpr (W == 1)
                        res = claim_bucket(reinterpret_cast<unsigned long long*>(keys), cnt, mask / BUCKET, K[u],
                                           (uint32_t)(h >> 32) & mask, nsl[u]);
                    else
                        res = claim_cas(reinterpret_cast<U128*>(keys), cnt, mask, K[u], (uint32_t)(h >> 32) & mask,
                                        nsl[u]);
                    if (res < 0) { if (!bad) atomicMin(&s_bad, r); bad = true; }
                    else newm |= (uint32_t)res << u;
                }
            }
            {  // this round's new slots onto the list: one shared atomic per warp
                const uint32_t nn = __popc(newm);
                uint32_t x = nn;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                uint32_t lb = 0;
                if (lane == 31 && x) lb = atomicAdd(&s_nlist, x);
                lb = __shfl_sync(0xffffffffu, lb, 31) + x - nn;
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if ((newm >> u) & 1u) list[min(lb + __popc(newm & ((1u << u) - 1u)), S - 1)] = (uint16_t)nsl[u];
            }
#pragma unroll
            for (int u = 0; u < U; ++u) K[u] = N[u];
        }
        if (bad) s_fail = 1;
        __syncthreads();  // inserts done; every thread has read slot q
        if (tid == 0) {
            // group g + 3's entry into slot q (landed before the group's last
            // barrier), the index after it claimed
            copy_group(&s_grp[q], P, gi_pend, n1, ntot);
            gi_pend = g0 + atomicAdd(P.work, 1ull);
        }
        if (tid == 32) {
            const uint32_t t = s_nlist;
            if (t > fill_cap) s_fail = 1;  // more than 7/8 full: split the group
            if (!filtered && !s_fail) s_obase = t ? atomicAdd(&P.ctr[P2C_OUT], (unsigned long long)t) : 0;
        }
        __syncthreads();
        if (s_fail) {
            // clear the table; the group comes back as two halves
            const uint32_t nl = min(s_nlist, S);
            for (uint32_t i = tid; i < nl; i += COUNT_THREADS) { keys[list[i]] = O::empty(); cnt[list[i]] = 0; }
            if (tid == 0) {
                Group f = g;
                if (g.parts < MAX_PARTS) {
                    // split into F key-hash parts: enough for half-full tables when the
                    // group ran to its end (its distinct keys are known), else 4
                    // distinct keys of the group: known when it ran to its end; else
                    // estimated from the keys seen before the table filled
                    uint64_t est = s_nlist;
                    if (s_bad != ~0u) {
                        const uint64_t hk = g.hi - g.lo;
                        uint64_t seen = (uint64_t)(s_bad + 1) * RK;
                        if (seen > hk) seen = hk;
                        est = (uint64_t)s_nlist * hk / (seen ? seen : 1);
                    }
                    const uint64_t need = (est + S / 2 - 1) / (S / 2);
                    uint32_t F = 2;
                    while (F < need) F <<= 1;
                    while (g.parts * F > MAX_PARTS) F >>= 1;
                    const unsigned long long i = atomicAdd(P.n_retry, (unsigned long long)F);
                    f.parts = F * g.parts;
                    if (i + F - 1 < P.retry_cap) {
                        for (uint32_t jf = 0; jf < F; ++jf) {
                            f.part = g.part + jf * g.parts;
                            P.retry[i + jf] = f;
                        }
                    }
                } else {
                    const unsigned long long i = atomicAdd(&P.ctr[P2C_FALLBACK], 1ull);
                    if (i < P.fallback_cap) P.fallback[i] = f;
                }
            }
        } else if (!filtered) {
            // ---- output: the listed slots in list order, pair i of the group to out[base + i]
            const uint32_t nl = s_nlist;
            const unsigned long long ob = s_obase;
            for (uint32_t i = tid; i < nl; i += COUNT_THREADS) {
                const uint32_t sl = list[i];
                const unsigned long long oi = ob + i;
                const uint32_t c = cnt[sl];
                if (oi < P.out_cap) {
                    O::store(P.out_keys, oi, keys[sl]);
                    P.out_counts[oi] = c + 1;
                    if (P.out_sample) P.out_sample[oi] = g.sample;
                }
                keys[sl] = O::empty();
                if (c) cnt[sl] = 0;
            }
            if (tid == 0) distinct += nl;
        } else {
            // ---- output: thread t owns slots t + j * COUNT_THREADS (a warp's accesses
            // are consecutive); per warp and round j one ballot places the kept
            // keys contiguously
            uint32_t keepm = 0, nocc = 0;
#pragma unroll
            for (uint32_t j = 0; j < SPT; ++j) {
                const uint32_t sl = tid + j * COUNT_THREADS;
                const bool occ = !O::is_empty(keys[sl]);
                nocc += occ ? 1u : 0u;
                bool keep = occ;
                if (filtered && occ) {
                    const uint32_t c = cnt[sl] + 1;
                    keep = (uint64_t)c >= P.ci && (uint64_t)c <= P.cx;
                }
                keepm |= (keep ? 1u : 0u) << j;
            }
            uint32_t wtot = 0;
#pragma unroll
            for (uint32_t j = 0; j < SPT; ++j) wtot += __popc(__ballot_sync(0xffffffffu, (keepm >> j) & 1u));
            nocc = __reduce_add_sync(0xffffffffu, nocc);
            if (lane == 0) { s_wout[wid] = wtot; distinct += nocc; }
            __syncthreads();
            if (wid == 0) {
                const uint32_t v = lane < COUNT_THREADS / 32 ? s_wout[lane] : 0u;
                uint32_t x = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane < COUNT_THREADS / 32) s_wout[lane] = x - v;
                if (lane == 31) s_obase = x ? atomicAdd(&P.ctr[P2C_OUT], (unsigned long long)x) : 0;
            }
            __syncthreads();
            unsigned long long o = s_obase + s_wout[wid];
#pragma unroll
            for (uint32_t j = 0; j < SPT; ++j) {
                const uint32_t sl = tid + j * COUNT_THREADS;
                const bool keep = (keepm >> j) & 1u;
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const unsigned long long i = o + __popc(bal & ((1u << lane) - 1));
                    if (i < P.out_cap) {
                        O::store(P.out_keys, i, keys[sl]);
                        P.out_counts[i] = cnt[sl] + 1;
                        if (P.out_sample) P.out_sample[i] = g.sample;
                    }
                }
                keys[sl] = O::empty();
                cnt[sl] = 0;
                o += __popc(bal);
            }
        }
        __syncthreads();  // every thread is done with the list
        if (tid == 0) {
            s_fail = 0;
            s_bad = ~0u;
            s_nlist = 0;
            asm volatile("cp.async.wait_all;" ::: "memory");  // group g + 3's entry has landed
        }
        __syncthreads();
    }
    if (lane == 0 && distinct) atomicAdd(&P.ctr[P2C_DISTINCT], distinct);
}

// ---------------------------------------------------------------- fallback
// A key range (one key-hash part of it) that did not fit in shared memory,
// counted in a global table of S slots (power of two >= 2 x the range).
template <int W>
__global__ void k_fb_insert(FallbackParams F) {
    using O = KeyOps<W>;
    auto* tk = reinterpret_cast<typename O::Key*>(F.tkeys);
    const auto* src = reinterpret_cast<const typename O::Key*>(F.keys);
    for (unsigned long long i = F.lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < F.hi;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const typename O::Key key = src[i];
        if (key_part<W>(key, F.parts) != F.part) continue;
        if (!tbl_add<W>(tk, F.tcnt, F.mask, key, F.mask + 1)) atomicExch(F.fail, 1u);
    }
}

template <int W>
__global__ void k_fb_init(void* keys, uint32_t* cnt, uint64_t S) {
    using O = KeyOps<W>;
    auto* kk = reinterpret_cast<typename O::Key*>(keys);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < S; i += (uint64_t)gridDim.x * blockDim.x) {
        kk[i] = O::empty();
        cnt[i] = 0;
    }
}

// Write the occupied slots that pass ci/cx (warp-aggregated output atomics).
template <int W>
__global__ void __launch_bounds__(256) k_fb_extract(const void* keys, const uint32_t* cnt, uint64_t S,
                                                    CountParams P, uint32_t sample) {
    using O = KeyOps<W>;
    const auto* kk = reinterpret_cast<const typename O::Key*>(keys);
    const int lane = threadIdx.x & 31;
    unsigned long long distinct = 0;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < S; i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + threadIdx.x;
        bool occ = false, keep = false;
        typename O::Key key;
        uint32_t c = 0;
        if (i < S) {
            key = kk[i];
            occ = !O::is_empty(key);
            if (occ) {
                c = cnt[i];
                keep = (uint64_t)c >= P.ci && (uint64_t)c <= P.cx;
            }
        }
        distinct += occ ? 1 : 0;
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (!bal) continue;
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&P.ctr[P2C_OUT], (unsigned long long)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (keep) {
            const uint64_t o = base + __popc(bal & ((1u << lane) - 1));
            if (o < P.out_cap) {
                O::store(P.out_keys, o, key);
                P.out_counts[o] = c;
                if (P.out_sample) P.out_sample[o] = sample;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) distinct += __shfl_down_sync(0xffffffffu, distinct, o);
    if (lane == 0 && distinct) atomicAdd(&P.ctr[P2C_DISTINCT], distinct);
}

// ---------------------------------------------------------------- sample-major output
// Jobs of several samples: the pairs, in group order, go sample-major so that
// each sample's pairs are one range. The pairs of one group are contiguous and
// of one sample, so the lanes of a warp nearly always share a sample: one
// atomic per distinct sample in the warp (match_any).
__global__ void k_samp_hist(const uint32_t* __restrict__ samp, uint64_t n, uint32_t* __restrict__ hist) {
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + threadIdx.x;
        const uint32_t s = i < n ? samp[i] : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xffffffffu, s);
        if (s != 0xFFFFFFFFu && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[s], (uint32_t)__popc(peers));
    }
}

template <int W>
__global__ void k_samp_scatter(const void* __restrict__ keys, const uint32_t* __restrict__ cnt,
                               const uint32_t* __restrict__ samp, uint64_t n, unsigned long long* __restrict__ cur,
                               void* __restrict__ keys2, uint32_t* __restrict__ cnt2) {
    using O = KeyOps<W>;
    const int lane = threadIdx.x & 31;
    const auto* kk = static_cast<const typename O::Key*>(keys);
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + threadIdx.x;
        const uint32_t s = i < n ? samp[i] : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xffffffffu, s);
        const int leader = __ffs(peers) - 1;
        unsigned long long base = 0;
        if (s != 0xFFFFFFFFu && lane == leader) base = atomicAdd(&cur[s], (unsigned long long)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (s != 0xFFFFFFFFu) {
            const uint64_t o = base + __popc(peers & ((1u << lane) - 1));
            O::store(keys2, o, kk[i]);
            cnt2[o] = cnt[i];
        }
    }
}

// ---------------------------------------------------------------- host side
size_t key_bytes(int W) { return W == 1 ? 8 : 16; }

// Table slots of a k_count CTA: the largest power of two whose keys and counts
// fit in one SM's shared memory (large tables mean large groups, and fewer of
// them to set up and drain).
uint32_t count_slots(int W) { return W == 1 ? 16384 : 8192; }

static size_t count_smem_bytes(int W, uint32_t slots) {
    if (W == 1) { CountSmem<1> L; L.layout(slots); return L.total; }
    CountSmem<2> L;
    L.layout(slots);
    return L.total;
}

namespace {
struct Carve {
    uint8_t* base;
    size_t off, cap;
    bool ok;
    template <class T>
    T* take(size_t n) {
        off = (off + 255) & ~size_t(255);
        if (off + n * sizeof(T) > cap) { ok = false; return nullptr; }
        T* p = reinterpret_cast<T*>(base + off);
        off += n * sizeof(T);
        return p;
    }
};

constexpr uint32_t NBIN_ALL = 1u << BIN_BITS;

struct P2Plan {
    uint64_t n_slices = 0, groups_cap = 0, retry_cap = 0, n_keys_alloc = 0, nsum = 0;
    std::vector<Slice> slices;
};

P2Plan make_plan(const P2Input& in) {
    P2Plan L;
    for (uint32_t c = 0; c < in.n_lists; ++c) {
        const uint64_t nd = std::min<uint64_t>(in.n_desc[c], in.desc_cap);
        for (uint64_t s = 0; s < nd; s += SLICE_DESC) {
            Slice sl;
            sl.r_lo = (uint64_t)c * in.desc_cap + s;
            sl.r_hi = (uint64_t)c * in.desc_cap + std::min<uint64_t>(nd, s + SLICE_DESC);
            L.slices.push_back(sl);
        }
    }
    L.n_slices = L.slices.size();
    // a segment of K keys has fewer than 2 K / target + 1 groups (two neighbouring
    // groups of k_plan hold more than `target` keys together)
    const uint64_t target = std::max<uint64_t>(1, (uint64_t)count_slots(in.W) * in.group_pct / 100);
    L.groups_cap = 2 * in.n_kmers / target + in.n_segs + 1;
    L.retry_cap = std::max<uint64_t>(4096, 2 * L.groups_cap);
    L.n_keys_alloc = in.n_kmers + 1;
    L.nsum = (NBIN_ALL + 8191) / 8192 + 2;
    return L;
}

// The scratch regions of one run, in order (the same walk sizes and places them).
struct P2Regions {
    unsigned long long* ctr;
    unsigned long long* aux;  // [0..1] retry counters, [2..3] list sizes of a retry pass
    unsigned long long* work; // [0..15] group counters of the first pass's launches, [16] of a retry pass
    unsigned long long* kofs;
    uint32_t* gfirst;
    unsigned long long* sums;
    Segment* segs;
    Slice* slices;
    Group* normal;
    Group* heavy;
    Group* retry[2];
    Group* fb;
    unsigned long long* scur;  // [n_samples] cursors of the sample-major copy
    uint8_t* keys;
};

P2Regions carve(Carve& c, const P2Input& in, const P2Plan& L) {
    P2Regions R;
    R.ctr = c.take<unsigned long long>(P2C_COUNT);
    R.aux = c.take<unsigned long long>(4);
    R.work = c.take<unsigned long long>(17);
    R.kofs = c.take<unsigned long long>(NBIN_ALL + 1);
    R.gfirst = c.take<uint32_t>(NBIN_ALL);
    R.sums = c.take<unsigned long long>(L.nsum);
    R.segs = c.take<Segment>(in.n_segs + 1);
    R.slices = c.take<Slice>(L.n_slices + 1);
    R.normal = c.take<Group>(L.groups_cap);
    R.heavy = c.take<Group>(L.groups_cap);
    R.retry[0] = c.take<Group>(L.retry_cap);
    R.retry[1] = c.take<Group>(L.retry_cap);
    R.fb = c.take<Group>(FALLBACK_CAP);
    R.scur = c.take<unsigned long long>(in.n_samples + 1);
    R.keys = c.take<uint8_t>(L.n_keys_alloc * key_bytes(in.W));
    return R;
}
}  // namespace

SampleBins layout_bins(const std::vector<unsigned long long>& sample_start, uint32_t seg_bins) {
    SampleBins B;
    B.start = sample_start;
    const size_t n = sample_start.size() - 1;
    const double total = (double)std::max<unsigned long long>(1, sample_start[n] - sample_start[0]);
    B.base.resize(n);
    B.bits.resize(n);
    // 2^bits <= the sample's share of `budget` bins (at least one bin)
    auto assign = [&](double budget) {
        uint64_t used = 0;
        for (size_t i = 0; i < n; ++i) {
            const double share = budget * (double)(sample_start[i + 1] - sample_start[i]) / total;
            uint32_t b = 0;
            while (b < BIN_BITS && (double)(2ull << b) <= share) ++b;
            B.bits[i] = (uint8_t)b;
            B.base[i] = (uint32_t)used;
            used += 1ull << b;
        }
        return used;
    };
    if (assign((double)NBIN_ALL) > NBIN_ALL) assign((double)(NBIN_ALL - n));  // one bin set aside per sample
    seg_bins = std::max<uint32_t>(1, seg_bins);
    for (size_t i = 0; i < n; ++i) {
        const uint32_t hi = B.base[i] + (1u << B.bits[i]);
        for (uint32_t lo = B.base[i]; lo < hi; lo += seg_bins) {
            Segment sg;
            sg.bin_lo = lo;
            sg.bin_hi = std::min(hi, lo + seg_bins);
            sg.sample = (uint32_t)i;
            sg.pad = 0;
            B.segs.push_back(sg);
        }
    }
    return B;
}

size_t phase2_scratch_bytes(const P2Input& in) {
    const P2Plan L = make_plan(in);
    Carve c{nullptr, 0, ~size_t(0), true};
    carve(c, in, L);
    return c.off + 256;
}

#define P2_CK(call, what)                                            \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            err = std::string(what) + ": " + cudaGetErrorString(e_); \
            return TG_ERR_CUDA;                                      \
        }                                                            \
    } while (0)

// Small counter reads (see OVERLAP_WORDS): src[0, n) to the mapped host words
// dst (device address), fenced for the host.
__global__ void k_peek(const unsigned long long* __restrict__ a, uint32_t na, const unsigned long long* __restrict__ b,
                       uint32_t nb, unsigned long long* dst) {
    const uint32_t i = threadIdx.x;
    if (i < na) dst[i] = a[i];
    else if (i < na + nb) dst[i] = b[i - na];
    __threadfence_system();
}

// Reads na counters at a and nb at b into out (host), then waits for the
// stream. With mapped words (ov.wave_out_dev) a kernel stores them there;
// otherwise cudaMemcpyAsync.
static cudaError_t read_counters(const P2Overlap& ov, const unsigned long long* a, uint32_t na,
                                 const unsigned long long* b, uint32_t nb, unsigned long long* out, cudaStream_t st) {
    if (ov.wave_out && ov.wave_out_dev && na + nb <= OVERLAP_WORDS - 16) {
        k_peek<<<1, 32, 0, st>>>(a, na, b, nb, ov.wave_out_dev + 16);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        const volatile unsigned long long* w = ov.wave_out + 16;
        for (uint32_t i = 0; i < na + nb; ++i) out[i] = w[i];
        return cudaSuccess;
    }
    cudaError_t e = cudaMemcpyAsync(out, a, 8 * (size_t)na, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nb) e = cudaMemcpyAsync(out + na, b, 8 * (size_t)nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

tg_status phase2_run(const P2Input& in, void* scratch, size_t scratch_cap, P2Output& out,
                     const std::function<void*(size_t)>& fallback_table, cudaStream_t st, cudaEvent_t ev_keys,
                     int* launches, std::string& err, const P2Overlap& ov) {
    const P2Plan L = make_plan(in);
    const int W = in.W;
    Carve c{static_cast<uint8_t*>(scratch), 0, scratch_cap, true};
    const P2Regions R = carve(c, in, L);
    if (!c.ok) { err = "phase-2 scratch too small"; return TG_ERR_OOM; }
    const uint32_t slots = count_slots(W);

    P2_CK(cudaMemsetAsync(R.ctr, 0, P2C_COUNT * 8, st), "memset");
    if (L.n_slices)
        P2_CK(cudaMemcpyAsync(R.slices, L.slices.data(), L.n_slices * sizeof(Slice), cudaMemcpyHostToDevice, st),
              "h2d");
    P2_CK(cudaMemcpyAsync(R.segs, in.segs, (size_t)in.n_segs * sizeof(Segment), cudaMemcpyHostToDevice, st), "h2d");
    // k-mer counts per bin -> first key of each bin (of this run's bins)
    P2_CK(launch_scan(in.binhist + in.bin_lo, in.bin_hi - in.bin_lo, R.kofs + in.bin_lo, R.sums, R.kofs + in.bin_hi,
                      st, launches),
          "scan");

    KeysParams K{};
    K.packed = in.packed;
    K.desc = in.desc;
    K.slices = R.slices;
    K.kofs = R.kofs;
    K.gfirst = R.gfirst;
    K.segs = R.segs;
    K.n_segs = in.n_segs;
    K.target = std::max<uint32_t>(1, slots * in.group_pct / 100);  // as in make_plan
    K.k = in.k;
    K.keys = R.keys;
    K.groups[0] = R.normal;
    K.groups[1] = R.heavy;
    K.groups_cap = L.groups_cap;
    K.ctr = R.ctr;
    K.bin_lo = in.bin_lo;
    K.bin_hi = in.bin_hi;
    {
        const uint32_t warps = PLAN_THREADS / 32;
        k_plan<<<(in.n_segs + warps - 1) / warps, PLAN_THREADS, 0, st>>>(K);  // before k_keys moves the cursors
    }
    P2_CK(cudaGetLastError(), "k_plan");
    ++*launches;
    if (L.n_slices) {
        // Large jobs: two launches, each writing the keys of half of the bins.
        // A record's keys land at its group's cursor; with every group open at
        // once fewer of the partly written sectors stay in L2 until their
        // neighbours fill them; with half of them open more do (3.1 G keys, bin
        // cursors: 28.0 -> 23.4 ms, four launches 25.1, eight 39.4; group
        // cursors: one launch 22.9, two 19.8), though every launch reads all
        // descriptors.
        const uint32_t KP = in.n_kmers > (1ull << 28) ? 2 : 1;
        const uint32_t span = in.bin_hi - in.bin_lo;
        for (uint32_t kp = 0; kp < KP; ++kp) {
            KeysParams Kp = K;
            Kp.bin_lo = in.bin_lo + (uint32_t)((uint64_t)span * kp / KP);
            Kp.bin_hi = in.bin_lo + (uint32_t)((uint64_t)span * (kp + 1) / KP);
            if (W == 1) k_keys<1><<<(unsigned)L.n_slices, P2_THREADS, 0, st>>>(Kp);
            else k_keys<2><<<(unsigned)L.n_slices, P2_THREADS, 0, st>>>(Kp);
            P2_CK(cudaGetLastError(), "k_keys");
            ++*launches;
        }
    }
    if (ev_keys) P2_CK(cudaEventRecord(ev_keys, st), "event");

    CountParams Q{};
    Q.keys = R.keys;
    Q.list[0] = R.normal;
    Q.list[1] = R.heavy;
    Q.n_list = R.ctr + P2C_NORMAL;  // [0] normal, [1] heavy: the heavy groups go first
    Q.fallback = R.fb;
    Q.fallback_cap = FALLBACK_CAP;
    Q.ci = in.ci;
    Q.cx = in.cx;
    Q.out_keys = out.keys;
    Q.out_counts = out.counts;
    Q.out_sample = out.samples;
    Q.out_cap = out.cap;
    Q.ctr = R.ctr;
    Q.retry_cap = L.retry_cap;
    Q.smem_slots = slots;
    const size_t sm = count_smem_bytes(W, slots);
    if (W == 1)
        P2_CK(set_smem_cap(k_count<1>, sm), "smem");
    else
        P2_CK(set_smem_cap(k_count<2>, sm), "smem");
    unsigned long long h[P2C_COUNT];
    // the groups of the first pass: their number is known once k_plan has run
    P2_CK(cudaMemcpyAsync(h, R.ctr, sizeof h, cudaMemcpyDeviceToHost, st), "d2h");
    P2_CK(cudaStreamSynchronize(st), "phase 2");
    if (h[P2C_NORMAL] > L.groups_cap || h[P2C_HEAVY] > L.groups_cap) {
        err = "group list overflow";
        return TG_ERR_TABLE;
    }
    const unsigned long long ngroups = h[P2C_NORMAL] + h[P2C_HEAVY];
    const uint32_t waves = ov.on_range && ov.wave_out && ov.wave_ev ? std::max<uint32_t>(1, std::min(ov.waves, 16u)) : 1;
    P2_CK(cudaMemsetAsync(R.work, 0, 8 * 17, st), "memset");
    uint64_t done = 0;  // output keys already handed to on_range
    for (int pass = 0;; ++pass) {
        // pass p writes its split groups to retry[p & 1]; pass p + 1 counts them
        Q.retry = R.retry[pass & 1];
        Q.n_retry = R.aux + (pass & 1);
        P2_CK(cudaMemsetAsync(Q.n_retry, 0, 8, st), "memset");
        // the first pass in `waves` launches over slices of the group sequence;
        // each slice's output range goes to on_range as soon as it is final
        const uint32_t nw = pass == 0 ? waves : 1;
        for (uint32_t wv = 0; wv < nw; ++wv) {
            Q.g_begin = pass == 0 ? ngroups * wv / nw : 0;
            Q.g_end = pass == 0 ? ngroups * (wv + 1) / nw : ~0ull;
            Q.work = R.work + (pass == 0 ? wv : 16);
            if (pass > 0) P2_CK(cudaMemsetAsync(Q.work, 0, 8, st), "memset");
            if (W == 1) k_count<1><<<in.n_sm * COUNT_PER_SM, COUNT_THREADS, sm, st>>>(Q);
            else k_count<2><<<in.n_sm * COUNT_PER_SM, COUNT_THREADS, sm, st>>>(Q);
            P2_CK(cudaGetLastError(), "k_count");
            ++*launches;
            if (nw > 1) {
                if (ov.wave_out_dev) k_peek<<<1, 32, 0, st>>>(R.ctr + P2C_OUT, 1, nullptr, 0, ov.wave_out_dev + wv);
                else P2_CK(cudaMemcpyAsync(ov.wave_out + wv, R.ctr + P2C_OUT, 8, cudaMemcpyDeviceToHost, st), "d2h");
                P2_CK(cudaEventRecord(ov.wave_ev[wv], st), "event");
            }
        }
        if (nw > 1) {
            for (uint32_t wv = 0; wv < nw; ++wv) {
                P2_CK(cudaEventSynchronize(ov.wave_ev[wv]), "wave");
                const uint64_t hi = std::min<uint64_t>(*(const volatile unsigned long long*)(ov.wave_out + wv), out.cap);
                if (hi > done) {
                    const tg_status rs = ov.on_range(done, hi);
                    if (rs != TG_OK) { err = "result copy failed"; return rs; }
                    done = hi;
                }
            }
        }
        unsigned long long hr[P2C_COUNT + 1];
        P2_CK(read_counters(ov, Q.n_retry, 1, R.ctr, P2C_COUNT, hr, st), "phase 2");
        const unsigned long long nret = hr[0];
        for (int c = 0; c < P2C_COUNT; ++c) h[c] = hr[c + 1];
        if (nret > L.retry_cap) { err = "too many groups to split"; return TG_ERR_TABLE; }
        if (nret == 0) break;
        const unsigned long long nl[2] = {0, nret};
        P2_CK(cudaMemcpyAsync(R.aux + 2, nl, 16, cudaMemcpyHostToDevice, st), "h2d");
        Q.list[0] = Q.list[1] = R.retry[pass & 1];
        Q.n_list = R.aux + 2;
    }
    out.fallback_groups = h[P2C_FALLBACK];
    // ---- key ranges that did not fit in shared memory
    if (h[P2C_FALLBACK] > 0) {
        if (h[P2C_FALLBACK] > FALLBACK_CAP) { err = "too many overflowing groups"; return TG_ERR_TABLE; }
        std::vector<Group> fl(h[P2C_FALLBACK]);
        P2_CK(cudaMemcpyAsync(fl.data(), R.fb, fl.size() * sizeof(Group), cudaMemcpyDeviceToHost, st), "d2h");
        P2_CK(cudaStreamSynchronize(st), "d2h");
        for (const Group& g : fl) {
            uint64_t S = 1024;
            while (S < 2 * (g.hi - g.lo) + 2) S <<= 1;
            if (S > (1ull << 32)) { err = "fallback table too large"; return TG_ERR_TABLE; }
            const size_t kbytes = (size_t)S * key_bytes(W);
            uint8_t* tab = static_cast<uint8_t*>(fallback_table(kbytes + (size_t)S * 4 + 16));
            if (!tab) { err = "no room for the fallback table"; return TG_ERR_OOM; }
            FallbackParams F{};
            F.keys = R.keys;
            F.lo = g.lo;
            F.hi = g.hi;
            F.parts = g.parts;
            F.part = g.part;
            F.sample = g.sample;
            F.tkeys = tab;
            F.tcnt = reinterpret_cast<uint32_t*>(tab + kbytes);
            F.mask = (uint32_t)(S - 1);
            F.fail = reinterpret_cast<uint32_t*>(tab + kbytes + (size_t)S * 4);
            P2_CK(cudaMemsetAsync(F.fail, 0, 4, st), "memset");
            const unsigned grid = (unsigned)in.n_sm * 4;
            if (W == 1) {
                k_fb_init<1><<<grid, 256, 0, st>>>(F.tkeys, F.tcnt, S);
                k_fb_insert<1><<<grid, 256, 0, st>>>(F);
                k_fb_extract<1><<<grid, 256, 0, st>>>(F.tkeys, F.tcnt, S, Q, g.sample);
            } else {
                k_fb_init<2><<<grid, 256, 0, st>>>(F.tkeys, F.tcnt, S);
                k_fb_insert<2><<<grid, 256, 0, st>>>(F);
                k_fb_extract<2><<<grid, 256, 0, st>>>(F.tkeys, F.tcnt, S, Q, g.sample);
            }
            P2_CK(cudaGetLastError(), "fallback");
            *launches += 3;
            uint32_t failed = 0;
            P2_CK(cudaMemcpyAsync(&failed, F.fail, 4, cudaMemcpyDeviceToHost, st), "d2h");
            P2_CK(cudaStreamSynchronize(st), "fallback");
            if (failed) { err = "fallback table overflow"; return TG_ERR_TABLE; }
        }
        P2_CK(read_counters(ov, R.ctr, P2C_COUNT, nullptr, 0, h, st), "fallback");
    }
    out.n_out = h[P2C_OUT];
    if (ov.on_range && std::min<uint64_t>(out.n_out, out.cap) > done) {
        const tg_status rs = ov.on_range(done, std::min<uint64_t>(out.n_out, out.cap));
        if (rs != TG_OK) { err = "result copy failed"; return rs; }
    }
    out.distinct = h[P2C_DISTINCT];
    if (out.samples && out.n_samples > 1 && out.n_samples <= in.n_samples && out.keys2 && out.counts2 && out.sample_off) {
        // sample-major copy: per-sample totals, their scan, the scatter
        const uint64_t n = std::min<uint64_t>(out.n_out, out.cap);
        uint32_t* hist = reinterpret_cast<uint32_t*>(R.kofs);  // the bin offsets are no longer needed
        P2_CK(cudaMemsetAsync(hist, 0, 4 * (size_t)out.n_samples, st), "memset");
        const unsigned grid = (unsigned)in.n_sm * 8;
        k_samp_hist<<<grid, 256, 0, st>>>(out.samples, n, hist);
        P2_CK(cudaGetLastError(), "k_samp_hist");
        P2_CK(launch_scan(hist, out.n_samples, out.sample_off, R.sums, out.sample_off + out.n_samples, st, launches),
              "scan");
        unsigned long long* cur = R.scur;  // the offsets, copied, as cursors
        P2_CK(cudaMemcpyAsync(cur, out.sample_off, 8 * (size_t)out.n_samples, cudaMemcpyDeviceToDevice, st), "copy");
        if (out.reorder_after) P2_CK(cudaStreamWaitEvent(st, out.reorder_after, 0), "wait");
        if (W == 1) k_samp_scatter<1><<<grid, 256, 0, st>>>(out.keys, out.counts, out.samples, n, cur, out.keys2, out.counts2);
        else k_samp_scatter<2><<<grid, 256, 0, st>>>(out.keys, out.counts, out.samples, n, cur, out.keys2, out.counts2);
        P2_CK(cudaGetLastError(), "k_samp_scatter");
        *launches += 2;
        P2_CK(cudaStreamSynchronize(st), "sample order");
    }
    out.groups = h[P2C_NORMAL] + h[P2C_HEAVY];
    out.heavy_groups = h[P2C_HEAVY];
    if (out.n_out > out.cap) { err = "output capacity exceeded"; return TG_ERR_TABLE; }
    return TG_OK;
}

}  // namespace tg
