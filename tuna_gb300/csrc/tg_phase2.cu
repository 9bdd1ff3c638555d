// tg_phase2.cu — Phase 2 on the GPU: exact count of every canonical k-mer of
// every bucket record, ci/cx filter and compaction of the surviving pairs.
//
// Reference behaviour (paths relative to the reference project root):
//   walk a record's k-mers        src/count.hpp:71-175 (bases MSB-first, roll the
//                                 k-mer and its reverse complement)
//   canonical form                include/kache-hash/Kmer.hpp:446-456, :629-646
//                                 (min of k-mer and reverse complement, word order)
//   count += 1 per instance       src/count.hpp:81, Streaming_Kmer_Hash_Table::upsert
//   keep ci <= count <= cx        src/count.hpp:202, :250, :287
//
// One CTA takes one bucket at a time from a size-ordered queue. A bucket whose
// k-mer instances exceed what one shared-memory table holds is split by further
// bits of the minimizer hash (the "fine" field of each record header) into
// groups; records of a group share their minimizer's fine bits, so every
// occurrence of a k-mer lands in the same group. Each group is counted in a
// shared-memory open-addressing table (64-bit CAS insert for k <= 31, 128-bit
// CAS for k <= 63, u32 atomicAdd counts). A group whose distinct k-mers do not
// fit is left to the global-memory table of k_fb_insert.
#include "tg_internal.cuh"

namespace tg {

constexpr int P2_THREADS = 256;
constexpr uint32_t F_MAX = 1024;         // fine groups per bucket
constexpr uint32_t PROBE_LIMIT = 256;    // linear-probe steps before a group gives up

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

// Walk the k-mers of one bucket record and add each canonical k-mer.
template <int W>
__device__ __forceinline__ bool add_record(const uint32_t* rec, int k, typename KeyOps<W>::Key* keys,
                                           uint32_t* cnt, uint32_t mask, uint32_t limit) {
    const uint32_t hdr = rec[0];
    const uint32_t nk = hdr & 0xFFu;
    const uint32_t* wd = rec + 1;
    const uint32_t len = nk + (uint32_t)k - 1;
    const uint32_t nw = (len + 15) / 16;
    if constexpr (W == 1) {
        // first k bases (k <= 31 -> within the first two words)
        const uint64_t top = ((uint64_t)wd[0] << 32) | (nw > 1 ? wd[1] : 0u);
        const uint64_t kmask = (1ull << (2 * k)) - 1;
        uint64_t f = top >> (64 - 2 * k);
        uint64_t r = revcomp64(f, k);
        const int rsh = 2 * k - 2;
        for (uint32_t j = 0;; ++j) {
            const uint64_t key = f < r ? f : r;
            if (!tbl_add<1>(keys, cnt, mask, key, limit)) return false;
            if (j + 1 >= nk) break;
            const uint32_t p = (uint32_t)k + j;  // next base
            const uint32_t b = (wd[p >> 4] >> (30 - 2 * (p & 15))) & 3u;
            f = ((f << 2) | b) & kmask;
            r = (r >> 2) | ((uint64_t)(3u - b) << rsh);
        }
    } else {
        // 32 <= k <= 63: first k bases from up to four words
        uint64_t w01 = ((uint64_t)wd[0] << 32) | (nw > 1 ? wd[1] : 0u);
        uint64_t w23 = ((uint64_t)(nw > 2 ? wd[2] : 0u) << 32) | (nw > 3 ? wd[3] : 0u);
        // 128-bit value of bases 0..63, then shift right to keep the first k
        const int sh = 128 - 2 * k;  // 2..64
        K2 f;
        if (sh >= 64) { f.lo = w01 >> (sh - 64); f.hi = 0; }
        else { f.lo = (w23 >> sh) | (w01 << (64 - sh)); f.hi = w01 >> sh; }
        K2 r = revcomp128(f, k);
        const int top_bits = 2 * k - 64;  // bits of hi in use
        const uint64_t hmask = top_bits >= 64 ? ~0ull : ((1ull << top_bits) - 1);
        const int rsh = 2 * k - 2 - 64;  // bit of the incoming complement in hi (-2 for k = 32)
        for (uint32_t j = 0;; ++j) {
            const K2& c = k2_less(f, r) ? f : r;
            U128 key;
            key.lo = c.lo;
            key.hi = c.hi;
            if (!tbl_add<2>(keys, cnt, mask, key, limit)) return false;
            if (j + 1 >= nk) break;
            const uint32_t p = (uint32_t)k + j;
            const uint32_t b = (wd[p >> 4] >> (30 - 2 * (p & 15))) & 3u;
            f.hi = ((f.hi << 2) | (f.lo >> 62)) & hmask;
            f.lo = (f.lo << 2) | b;
            r.lo = (r.lo >> 2) | (r.hi << 62);
            if (rsh >= 0) r.hi = (r.hi >> 2) | ((uint64_t)(3u - b) << rsh);
            else r.lo |= (uint64_t)(3u - b) << 62;  // k = 32: the k-mer fills lo exactly
        }
    }
    return true;
}

template <int W>
struct P2Smem {
    size_t keys, cnt, gr, gk, gs, total;
    __host__ __device__ void layout(uint32_t slots) {
        size_t o = 0;
        keys = o; o += KeyOps<W>::BYTES * (size_t)slots;
        cnt = o; o += 4 * (size_t)slots;
        gr = o; o += 4 * (size_t)F_MAX;
        gk = o; o += 4 * (size_t)F_MAX;
        gs = o; o += 4 * (size_t)F_MAX;
        total = (o + 15) & ~size_t(15);
    }
};

// Write the occupied slots [0, S) that pass ci/cx to the output (warp-aggregated).
template <int W>
__device__ void extract(const typename KeyOps<W>::Key* keys, const uint32_t* cnt, uint32_t S,
                        const Phase2Params& P, unsigned long long& distinct) {
    using O = KeyOps<W>;
    const int lane = threadIdx.x & 31;
    const uint32_t iters = (S + P2_THREADS - 1) / P2_THREADS;
    for (uint32_t it = 0; it < iters; ++it) {
        const uint32_t i = it * P2_THREADS + threadIdx.x;
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

template <int W>
__global__ void __launch_bounds__(P2_THREADS)
k_count(Phase2Params P) {
    using O = KeyOps<W>;
    extern __shared__ __align__(16) uint8_t smem[];
    P2Smem<W> L;
    L.layout(P.smem_slots);
    typename O::Key* keys = reinterpret_cast<typename O::Key*>(smem + L.keys);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem + L.cnt);
    uint32_t* s_gr = reinterpret_cast<uint32_t*>(smem + L.gr);
    uint32_t* s_gk = reinterpret_cast<uint32_t*>(smem + L.gk);
    uint32_t* s_gs = reinterpret_cast<uint32_t*>(smem + L.gs);
    __shared__ uint32_t s_bucket;
    __shared__ uint32_t s_fail;
    __shared__ uint32_t s_scan[P2_THREADS / 32];

    const int tid = threadIdx.x;
    const uint32_t C = P.n_cta1;
    uint32_t* scratch = P.scratch + (uint64_t)blockIdx.x * P.scratch_cap;
    unsigned long long distinct = 0;

    for (;;) {
        if (tid == 0) s_bucket = atomicAdd(P.work, 1u);
        __syncthreads();
        const uint32_t qi = s_bucket;
        __syncthreads();
        if (qi >= P.n_buckets) break;
        const uint32_t b = P.order[qi];
        const uint64_t r0 = P.off_r[(uint64_t)b * C];
        const uint64_t r1 = P.off_r[(uint64_t)(b + 1) * C];  // off_r has a final total entry
        const uint64_t wb = P.off_w[(uint64_t)b * C];
        const uint32_t nrec = (uint32_t)(r1 - r0);
        if (nrec == 0) continue;
        const uint64_t K = P.bucket_kmers[b];
        uint32_t F = 1;
        while ((uint64_t)F * P.target < K && F < F_MAX && F < (1u << P.fine_bits)) F <<= 1;
        const uint32_t* recs = P.records + wb;
        const uint32_t* list = P.index + r0;
        if (F > 1) {
            for (uint32_t g = tid; g < F; g += P2_THREADS) { s_gr[g] = 0; s_gk[g] = 0; }
            __syncthreads();
            for (uint32_t i = tid; i < nrec; i += P2_THREADS) {
                const uint32_t hdr = recs[list[i]];
                const uint32_t g = (hdr >> 8) & (F - 1);
                atomicAdd(&s_gr[g], 1u);
                atomicAdd(&s_gk[g], hdr & 0xFFu);
            }
            __syncthreads();
            // exclusive scan of group record counts (F <= F_MAX, PER = F_MAX / P2_THREADS)
            {
                constexpr uint32_t PER = F_MAX / P2_THREADS;
                uint32_t loc[PER], acc = 0;
#pragma unroll
                for (uint32_t j = 0; j < PER; ++j) {
                    const uint32_t g = tid * PER + j;
                    loc[j] = g < F ? s_gr[g] : 0;
                    acc += loc[j];
                }
                // block scan of acc
                uint32_t x = acc;
                const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) s_scan[wid] = x;
                __syncthreads();
                if (wid == 0) {
                    uint32_t t = lane < P2_THREADS / 32 ? s_scan[lane] : 0;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                        if (lane >= o) t += y;
                    }
                    if (lane < P2_THREADS / 32) s_scan[lane] = t;
                }
                __syncthreads();
                uint32_t run = (wid ? s_scan[wid - 1] : 0) + x - acc;
#pragma unroll
                for (uint32_t j = 0; j < PER; ++j) {
                    const uint32_t g = tid * PER + j;
                    if (g < F) s_gs[g] = run;
                    run += loc[j];
                }
            }
            __syncthreads();
            // scatter record offsets by group into this CTA's scratch; s_gr
            // becomes the per-group cursor (restored below from s_gs)
            for (uint32_t g = tid; g < F; g += P2_THREADS) s_gr[g] = s_gs[g];
            __syncthreads();
            for (uint32_t i = tid; i < nrec; i += P2_THREADS) {
                const uint32_t off = list[i];
                const uint32_t hdr = recs[off];
                const uint32_t g = (hdr >> 8) & (F - 1);
                const uint32_t pos = atomicAdd(&s_gr[g], 1u);
                scratch[pos] = off;
            }
            __syncthreads();
            list = scratch;
        }
        for (uint32_t g = 0; g < F; ++g) {
            uint32_t gstart, gcount;
            uint64_t gk;
            if (F == 1) { gstart = 0; gcount = nrec; gk = K; }
            else {
                gstart = s_gs[g];
                gcount = s_gr[g] - s_gs[g];
                gk = s_gk[g];
            }
            if (gcount == 0) continue;
            uint32_t S = 256;
            while ((uint64_t)S < 2 * gk && S < P.smem_slots) S <<= 1;
            if (S > P.smem_slots) S = P.smem_slots;
            const uint32_t mask = S - 1;
            for (uint32_t i = tid; i < S; i += P2_THREADS) { keys[i] = O::empty(); cnt[i] = 0; }
            if (tid == 0) s_fail = 0;
            __syncthreads();
            const uint32_t limit = min(S, PROBE_LIMIT);
            for (uint32_t i = tid; i < gcount; i += P2_THREADS) {
                if (*reinterpret_cast<volatile uint32_t*>(&s_fail)) break;
                if (!add_record<W>(recs + list[gstart + i], P.k, keys, cnt, mask, limit)) {
                    s_fail = 1;
                    break;
                }
            }
            __syncthreads();
            if (s_fail) {
                if (tid == 0) {
                    const unsigned long long slot = atomicAdd(&P.out_n[2], 1ull);
                    if (slot < P.fallback_cap) {
                        P.fallback[3 * slot + 0] = b;
                        P.fallback[3 * slot + 1] = g;
                        P.fallback[3 * slot + 2] = F;
                    }
                }
                __syncthreads();
                continue;
            }
            extract<W>(keys, cnt, S, P, distinct);
            __syncthreads();
        }
    }
    for (int o = 16; o > 0; o >>= 1) distinct += __shfl_down_sync(0xffffffffu, distinct, o);
    if ((tid & 31) == 0 && distinct) atomicAdd(&P.out_n[1], distinct);
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
        const uint32_t* rec = P.records + P.wb + P.index[P.r0 + i];
        if (((rec[0] >> 8) & (P.F - 1)) != P.group) continue;
        if (!add_record<W>(rec, P.k, keys, P.cnt, P.mask, P.mask + 1)) atomicExch(P.fail, 1u);
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
__global__ void __launch_bounds__(P2_THREADS) k_fb_extract(const void* keys, const uint32_t* cnt, uint64_t S,
                                                            Phase2Params P) {
    using O = KeyOps<W>;
    const auto* kk = reinterpret_cast<const typename O::Key*>(keys);
    unsigned long long distinct = 0;
    const uint64_t chunk = (uint64_t)P2_THREADS * 64;
    for (uint64_t base = (uint64_t)blockIdx.x * chunk; base < S; base += (uint64_t)gridDim.x * chunk) {
        const uint32_t n = (uint32_t)((S - base) < chunk ? (S - base) : chunk);
        extract<W>(kk + base, cnt + base, n, P, distinct);
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
        k_fb_extract<1><<<grid, P2_THREADS, 0, st>>>(F.keys, F.cnt, S, P);
    } else {
        k_fb_init<2><<<grid, 256, 0, st>>>(F.keys, F.cnt, S);
        k_fb_insert<2><<<grid, 256, 0, st>>>(F);
        k_fb_extract<2><<<grid, P2_THREADS, 0, st>>>(F.keys, F.cnt, S, P);
    }
    *launches += 3;
    return cudaGetLastError();
}

}  // namespace tg
