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
// One CTA takes one bucket at a time from a size-ordered queue. A bucket whose
// k-mer instances exceed what one shared-memory table holds is split by further
// bits of the minimizer hash (each descriptor's bin) into groups of contiguous
// bins; all occurrences of a canonical k-mer share its minimizer, so they land
// in the same group. Each group is counted in a shared-memory open-addressing
// table (64-bit CAS insert for k <= 31, 128-bit CAS for k <= 63, u32 atomicAdd
// counts). A group that overflows is halved; a single bin that still overflows
// is left to the global-memory table of k_fb_insert.
#include "tg_internal.cuh"

namespace tg {

constexpr int P2_THREADS = 1024;
constexpr uint32_t NBINS = 1024;         // minimizer-bit bins per bucket for the group split
constexpr uint32_t PROBE_LIMIT = 128;    // linear-probe steps before a group is split
constexpr uint32_t MAX_PARTS = 4096;     // key-hash passes over one bin before the global table
constexpr int UNROLL = 4;                // k-mers per lane per round of k_count

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
    __device__ static void store_out(void* out, uint64_t i, const Key& k) {
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
    __device__ static void store_out(void* out, uint64_t i, const Key& k) {
        reinterpret_cast<U128*>(out)[i] = k;
    }
};

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

// Add one k-mer instance. Returns 1 and the slot when the key claimed a new
// slot (the caller appends it to the used list), 0 when the key was already
// present, -1 when `limit` probes found no place (the group must be split).
template <int W>
__device__ __forceinline__ int tbl_claim(typename KeyOps<W>::Key* keys, uint32_t* cnt, uint32_t mask,
                                         const typename KeyOps<W>::Key& key, uint32_t limit, uint32_t& slot) {
    using O = KeyOps<W>;
    uint32_t h = (uint32_t)(O::hash(key) >> 32) & mask;
    for (uint32_t p = 0; p < limit; ++p) {
        if constexpr (W == 1) {
            const typename O::Key cur = O::load(&keys[h]);
            if (O::eq(cur, key)) { atomicAdd(&cnt[h], 1u); return 0; }
            if (O::is_empty(cur)) {
                const typename O::Key prev = O::cas(&keys[h], O::empty(), key);
                if (O::is_empty(prev)) { atomicAdd(&cnt[h], 1u); slot = h; return 1; }
                if (O::eq(prev, key)) { atomicAdd(&cnt[h], 1u); return 0; }
            }
        } else {
            const typename O::Key prev = O::cas(&keys[h], O::empty(), key);
            if (O::is_empty(prev)) { atomicAdd(&cnt[h], 1u); slot = h; return 1; }
            if (O::eq(prev, key)) { atomicAdd(&cnt[h], 1u); return 0; }
        }
        h = (h + 1) & mask;
    }
    return -1;
}

template <int W>
struct P2Smem {
    size_t keys, cnt, used, brec, bkm, boff, pre, total;
    __host__ __device__ void layout(uint32_t slots) {
        size_t o = 0;
        keys = o; o += KeyOps<W>::BYTES * (size_t)slots;
        cnt = o; o += 4 * (size_t)slots;
        used = o; o += 2 * (size_t)slots;
        o = (o + 15) & ~size_t(15);
        brec = o; o += 4 * (size_t)NBINS;
        bkm = o; o += 4 * (size_t)NBINS;
        boff = o; o += 4 * (size_t)(NBINS + 1);
        o = (o + 15) & ~size_t(15);
        pre = o; o += 4 * (size_t)(NBINS + 1);
        total = (o + 15) & ~size_t(15);
    }
};

// Block-wide exclusive scan of a[0..n) (n <= 2 * P2_THREADS) into out[0..n],
// out[n] = total.
__device__ void scan_bins(const uint32_t* a, uint32_t n, uint32_t* out, uint32_t* s_warp) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t i0 = 2 * tid, i1 = 2 * tid + 1;
    const uint32_t v0 = i0 < n ? a[i0] : 0, v1 = i1 < n ? a[i1] : 0;
    const uint32_t v = v0 + v1;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < P2_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < P2_THREADS / 32) s_warp[lane] = t;
    }
    __syncthreads();
    const uint32_t before = (wid ? s_warp[wid - 1] : 0) + x - v;
    if (i0 < n) out[i0] = before;
    if (i1 < n) out[i1] = before + v0;
    if (tid == P2_THREADS - 1) out[n] = s_warp[P2_THREADS / 32 - 1];
    __syncthreads();
}

// One CTA per SM. The table is cleared once; each group adds its k-mers,
// writes the used slots that pass ci/cx, and resets only those slots.
//
// A warp takes 32 descriptors at a time and spreads their k-mers over its
// lanes: in each round lane t handles the warp's k-mer number r + t, whose
// descriptor is found by a search over the descriptors' inclusive k-mer
// prefix sums (five shuffles). All lanes stay busy whatever the record lengths.
template <int W>
__global__ void __launch_bounds__(P2_THREADS, 1)
k_count(Phase2Params P) {
    using O = KeyOps<W>;
    extern __shared__ __align__(16) uint8_t smem[];
    P2Smem<W> L;
    L.layout(P.smem_slots);
    typename O::Key* keys = reinterpret_cast<typename O::Key*>(smem + L.keys);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + L.cnt);
    uint16_t* used = reinterpret_cast<uint16_t*>(smem + L.used);
    uint32_t* brec = reinterpret_cast<uint32_t*>(smem + L.brec);
    uint32_t* bkm = reinterpret_cast<uint32_t*>(smem + L.bkm);
    uint32_t* boff = reinterpret_cast<uint32_t*>(smem + L.boff);
    uint32_t* pre = reinterpret_cast<uint32_t*>(smem + L.pre);
    __shared__ uint32_t s_bucket, s_next, s_fail, s_nused, s_sp;
    __shared__ uint32_t s_warp[P2_THREADS / 32];
    __shared__ uint4 s_stack[64];  // {first bin, end bin, key-hash parts J, part j}
    __shared__ unsigned long long s_obase;
    __shared__ uint32_t s_ocur;

    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t C = P.n_cta1;
    const uint32_t S = P.smem_slots, mask = S - 1;
    const uint32_t fill_cap = S - S / 8;  // a group is split beyond 7/8 occupancy
    const uint32_t bin_bits = 20 - P.p1_bits;
    const uint32_t nb = min(NBINS, 1u << bin_bits);
    const int k = P.k;
    uint64_t* scratch = P.scratch + (uint64_t)blockIdx.x * P.scratch_cap;
    unsigned long long distinct = 0;
    for (uint32_t i = tid; i < S; i += P2_THREADS) { keys[i] = O::empty(); cnt[i] = 0; }
    if (tid == 0) s_nused = 0;
    __syncthreads();

    for (;;) {
        if (tid == 0) s_bucket = atomicAdd(P.work, 1u);
        __syncthreads();
        const uint32_t qi = s_bucket;
        __syncthreads();
        if (qi >= P.n_buckets) break;
        const uint32_t b = P.order[qi];
        const uint64_t r0 = P.off_r[(uint64_t)b * C];
        const uint32_t nrec = (uint32_t)(P.off_r[(uint64_t)(b + 1) * C] - r0);
        if (nrec == 0) continue;
        const uint64_t* bd = P.bdesc + r0;
        const uint64_t K = P.bucket_kmers[b];
        bool binned = false;

        auto bin_of = [&](uint64_t d) -> uint32_t { return (desc_mlo(d) >> P.p1_bits) & (nb - 1); };
        auto bin_pass = [&]() {
            for (uint32_t i = tid; i < nb; i += P2_THREADS) { brec[i] = 0; bkm[i] = 0; }
            __syncthreads();
            for (uint32_t i = tid; i < nrec; i += P2_THREADS) {
                const uint64_t d = bd[i];
                const uint32_t bin = bin_of(d);
                atomicAdd(&brec[bin], 1u);
                atomicAdd(&bkm[bin], desc_nk(d));
            }
            __syncthreads();
            scan_bins(brec, nb, boff, s_warp);
            scan_bins(bkm, nb, pre, s_warp);
            for (uint32_t i = tid; i < nb; i += P2_THREADS) brec[i] = boff[i];
            __syncthreads();
            for (uint32_t i = tid; i < nrec; i += P2_THREADS) {
                const uint64_t d = bd[i];
                scratch[atomicAdd(&brec[bin_of(d)], 1u)] = d;
            }
            __syncthreads();
        };

        if (K > P.target) {
            bin_pass();
            binned = true;
        }
        if (tid == 0) { s_stack[0] = make_uint4(0, nb, 1, 0); s_sp = 1; }
        __syncthreads();
        while (s_sp > 0) {
            // ---- pop a bin range; halve it while it holds more k-mers than the target
            __syncthreads();
            if (tid == 0) {
                uint4 rg = s_stack[--s_sp];
                while (binned && rg.z == 1 && rg.y - rg.x > 1 && pre[rg.y] - pre[rg.x] > P.target && s_sp < 62) {
                    const uint32_t half = pre[rg.x] + (pre[rg.y] - pre[rg.x]) / 2;
                    uint32_t lo = rg.x + 1, hi = rg.y - 1;  // first bin m in (x, y) with pre[m] >= half
                    while (lo < hi) {
                        const uint32_t md = (lo + hi) / 2;
                        if (pre[md] >= half) hi = md; else lo = md + 1;
                    }
                    s_stack[s_sp++] = make_uint4(lo, rg.y, 1, 0);
                    rg.y = lo;
                }
                s_stack[63] = rg;  // the range to count now
                s_next = 0;
                s_fail = 0;
            }
            __syncthreads();
            const uint4 rg = s_stack[63];
            const uint32_t part_mask = rg.z - 1, part = rg.w;
            const uint64_t* list = binned ? scratch + boff[rg.x] : bd;
            const uint32_t cnt_r = binned ? boff[rg.y] - boff[rg.x] : nrec;
            // ---- add every k-mer of the range: batches of 32 descriptors per warp
            for (;;) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(&s_next, 32u);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= cnt_r) break;
                const uint32_t i = base + lane;
                const uint64_t d = i < cnt_r ? list[i] : 0;
                const uint32_t nk = i < cnt_r ? desc_nk(d) : 0;
                const uint64_t st = desc_start(d);
                uint32_t incl = nk;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                const uint32_t excl = incl - nk;
                const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                bool bad = false;
                // U k-mers per lane per round: their loads and probes overlap
                for (uint32_t t0 = 0; t0 < total; t0 += 32 * UNROLL) {
                    typename O::Key kv[UNROLL];
                    bool act[UNROLL];
#pragma unroll
                    for (int u = 0; u < UNROLL; ++u) {
                        const uint32_t t = t0 + 32 * u + lane;
                        // owner = first lane whose inclusive prefix exceeds t
                        uint32_t lo = 0;
#pragma unroll
                        for (uint32_t step = 16; step >= 1; step >>= 1) {
                            const uint32_t c = lo + step - 1;
                            const uint32_t v = __shfl_sync(0xffffffffu, incl, c);
                            if (v <= t) lo = c + 1;
                        }
                        const uint32_t owner = lo & 31;
                        const uint64_t ost = __shfl_sync(0xffffffffu, st, owner);
                        const uint32_t opre = __shfl_sync(0xffffffffu, excl, owner);
                        act[u] = t < total;
                        if (act[u]) kv[u] = kmer_key<W>(P.packed, ost + (t - opre), k);
                    }
#pragma unroll
                    for (int u = 0; u < UNROLL; ++u) {
                        int r = 0;
                        uint32_t slot = 0;
                        // a bin split by key hash counts only its part of the keys
                        if (act[u] && !bad && ((uint32_t)(O::hash(kv[u]) >> 8) & part_mask) == part) {
                            r = tbl_claim<W>(keys, cnt, mask, kv[u], PROBE_LIMIT, slot);
                            if (r < 0) bad = true;
                        }
                        // append the newly claimed slots to the used list, one atomic per warp
                        const unsigned nm = __ballot_sync(0xffffffffu, r > 0);
                        if (nm) {
                            uint32_t ub = 0;
                            if (lane == 0) ub = atomicAdd(&s_nused, (uint32_t)__popc(nm));
                            ub = __shfl_sync(0xffffffffu, ub, 0);
                            const uint32_t uu = ub + __popc(nm & ((1u << lane) - 1));
                            if (r > 0) {
                                used[uu] = (uint16_t)slot;      // uu < S: at most S slots can be claimed
                                if (uu >= fill_cap) bad = true;  // the table is 7/8 full: split the group
                            }
                        }
                    }
                }
                if (bad) *reinterpret_cast<volatile uint32_t*>(&s_fail) = 1;
                if (__any_sync(0xffffffffu, *reinterpret_cast<volatile uint32_t*>(&s_fail) != 0)) break;
            }
            __syncthreads();
            const uint32_t nu = min(s_nused, S);
            if (s_fail) {
                // reset the partial table, then split the range (or hand it to the global table)
                for (uint32_t i = tid; i < nu; i += P2_THREADS) { keys[used[i]] = O::empty(); cnt[used[i]] = 0; }
                __syncthreads();
                if (!binned) {
                    bin_pass();
                    binned = true;
                    if (tid == 0) { s_stack[0] = make_uint4(0, nb, 1, 0); s_sp = 1; }
                } else if (tid == 0) {
                    if (rg.y - rg.x > 1 && s_sp < 62) {
                        const uint32_t mid = (rg.x + rg.y) / 2;
                        s_stack[s_sp++] = make_uint4(mid, rg.y, 1, 0);
                        s_stack[s_sp++] = make_uint4(rg.x, mid, 1, 0);
                    } else if (rg.z < MAX_PARTS && s_sp < 62) {
                        // one bin with more distinct k-mers than a table: count it in
                        // 2J passes, each over the keys whose hash bits select it
                        s_stack[s_sp++] = make_uint4(rg.x, rg.y, 2 * rg.z, rg.w + rg.z);
                        s_stack[s_sp++] = make_uint4(rg.x, rg.y, 2 * rg.z, rg.w);
                    } else {
                        for (uint32_t g = rg.x; g < rg.y; ++g) {
                            const unsigned long long slot = atomicAdd(&P.out_n[2], 1ull);
                            if (slot < P.fallback_cap) {
                                P.fallback[3 * slot + 0] = b;
                                P.fallback[3 * slot + 1] = g;
                                P.fallback[3 * slot + 2] = nb;
                            }
                        }
                    }
                }
                if (tid == 0) s_nused = 0;
                __syncthreads();
                continue;
            }
            // ---- output the used slots that pass ci/cx, and reset them. One
            // global atomic per group reserves the output range; inside it each
            // warp claims a contiguous slice per pass, so its stores coalesce.
            uint32_t mine = 0;
            for (uint32_t i = tid; i < nu; i += P2_THREADS) {
                const uint32_t c = cnt[used[i]];
                mine += ((uint64_t)c >= P.ci && (uint64_t)c <= P.cx) ? 1u : 0u;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
            if (tid == 0) s_ocur = 0;
            if (lane == 0) s_warp[tid >> 5] = mine;
            __syncthreads();
            if (tid == 0) {
                uint32_t t = 0;
                for (int w2 = 0; w2 < P2_THREADS / 32; ++w2) t += s_warp[w2];
                if (t) s_obase = atomicAdd(&P.out_n[0], (unsigned long long)t);
            }
            __syncthreads();
            const unsigned long long obase = s_obase;
            const uint32_t iters = (nu + P2_THREADS - 1) / P2_THREADS;
            for (uint32_t it = 0; it < iters; ++it) {
                const uint32_t i = it * P2_THREADS + tid;
                bool keep = false;
                typename O::Key key;
                uint32_t c = 0;
                if (i < nu) {
                    const uint32_t sl = used[i];
                    key = keys[sl];
                    c = cnt[sl];
                    keep = (uint64_t)c >= P.ci && (uint64_t)c <= P.cx;
                    keys[sl] = O::empty();
                    cnt[sl] = 0;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (bal) {
                    uint32_t wb = 0;
                    if (lane == 0) wb = atomicAdd(&s_ocur, (uint32_t)__popc(bal));
                    wb = __shfl_sync(0xffffffffu, wb, 0);
                    if (keep) {
                        const uint64_t o = obase + wb + __popc(bal & ((1u << lane) - 1));
                        if (o < P.out_cap) {
                            O::store_out(P.out_keys, o, key);
                            P.out_counts[o] = c;
                        }
                    }
                }
            }
            if (tid == 0) { distinct += nu; s_nused = 0; }
            __syncthreads();
        }
    }
    if (tid == 0 && distinct) atomicAdd(&P.out_n[1], distinct);
}

// Write the occupied slots [0, S) of a global table that pass ci/cx (warp-aggregated).
template <int W>
__device__ void extract_all(const typename KeyOps<W>::Key* keys, const uint32_t* cnt, uint32_t S,
                            const Phase2Params& P, unsigned long long& distinct) {
    using O = KeyOps<W>;
    const int lane = threadIdx.x & 31;
    const uint32_t iters = (S + blockDim.x - 1) / blockDim.x;
    for (uint32_t it = 0; it < iters; ++it) {
        const uint32_t i = it * blockDim.x + threadIdx.x;
        bool occ = false, keep = false;
        typename O::Key key;
        uint32_t c = 0;
        if (i < S) {
            key = keys[i];
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
        if (lane == 0) base = atomicAdd(&P.out_n[0], (unsigned long long)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (keep) {
            const uint64_t o = base + __popc(bal & ((1u << lane) - 1));
            if (o < P.out_cap) {
                O::store_out(P.out_keys, o, key);
                P.out_counts[o] = c;
            }
        }
    }
}

// ---------------------------------------------------------------- fallback
// A group that overflowed its shared-memory table is counted in a global
// table of S slots (power of two >= 2 x its k-mer instances): every CTA walks a
// slice of the bucket's records and adds the k-mers of the group's records.

template <int W>
__global__ void k_fb_insert(FallbackParams P) {
    using O = KeyOps<W>;
    auto* keys = reinterpret_cast<typename O::Key*>(P.keys);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.nrec;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t d = P.bdesc[P.r0 + i];
        if (((desc_mlo(d) >> P.p1_bits) & (P.nbins - 1)) != P.bin) continue;
        const uint64_t st = desc_start(d);
        const uint32_t nk = desc_nk(d);
        for (uint32_t j = 0; j < nk; ++j)
            if (!tbl_add<W>(keys, P.cnt, P.mask, kmer_key<W>(P.packed, st + j, P.k), P.mask + 1))
                atomicExch(P.fail, 1u);
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

template <int W>
__global__ void __launch_bounds__(256) k_fb_extract(const void* keys, const uint32_t* cnt, uint64_t S,
                                                            Phase2Params P) {
    using O = KeyOps<W>;
    const auto* kk = reinterpret_cast<const typename O::Key*>(keys);
    unsigned long long distinct = 0;
    const uint64_t chunk = (uint64_t)256 * 64;
    for (uint64_t base = (uint64_t)blockIdx.x * chunk; base < S; base += (uint64_t)gridDim.x * chunk) {
        const uint32_t n = (uint32_t)((S - base) < chunk ? (S - base) : chunk);
        extract_all<W>(kk + base, cnt + base, n, P, distinct);
    }
    for (int o = 16; o > 0; o >>= 1) distinct += __shfl_down_sync(0xffffffffu, distinct, o);
    if ((threadIdx.x & 31) == 0 && distinct) atomicAdd(&P.out_n[1], distinct);
}

// ---------------------------------------------------------------- launchers
size_t count_smem_bytes(int W, uint32_t slots) {
    if (W == 1) { P2Smem<1> L; L.layout(slots); return L.total; }
    P2Smem<2> L;
    L.layout(slots);
    return L.total;
}

size_t key_bytes(int W) { return W == 1 ? 8 : 16; }

cudaError_t launch_count(int W, const Phase2Params& P, uint32_t grid, cudaStream_t st) {
    const size_t sm = count_smem_bytes(W, P.smem_slots);
    cudaError_t e;
    if (W == 1) {
        e = cudaFuncSetAttribute(k_count<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_count<1><<<grid, P2_THREADS, sm, st>>>(P);
    } else {
        e = cudaFuncSetAttribute(k_count<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_count<2><<<grid, P2_THREADS, sm, st>>>(P);
    }
    return cudaGetLastError();
}

cudaError_t launch_fallback(int W, const FallbackParams& F, uint64_t S, const Phase2Params& P, uint32_t grid,
                            cudaStream_t st, int* launches) {
    if (W == 1) {
        k_fb_init<1><<<grid, 256, 0, st>>>(F.keys, F.cnt, S);
        k_fb_insert<1><<<grid, 256, 0, st>>>(F);
        k_fb_extract<1><<<grid, 256, 0, st>>>(F.keys, F.cnt, S, P);
    } else {
        k_fb_init<2><<<grid, 256, 0, st>>>(F.keys, F.cnt, S);
        k_fb_insert<2><<<grid, 256, 0, st>>>(F);
        k_fb_extract<2><<<grid, 256, 0, st>>>(F.keys, F.cnt, S, P);
    }
    *launches += 3;
    return cudaGetLastError();
}

}  // namespace tg
