// tg_phase1.cu — Phase 1 on the GPU: 2-bit packing, superkmer cutting and the
// bucketing of superkmer record descriptors in HBM.
//
// Reference behaviour (paths relative to the reference project root):
//   ASCII -> kache 2-bit          src/partition_hash.hpp:68-70
//   canonical ntHash per m-mer    include/nt_hash.hpp:74-124
//   minimizer of each k-mer       include/minimizer_window.hpp (value = min over
//                                 the k-m+1 m-mer hashes of the k-mer)
//   superkmer boundaries          src/partition_hash.hpp:78-93: a new record at
//                                 a minimizer change, or when the record would
//                                 exceed hdr_t::max bases
//   partition of a record         src/partition_hash.hpp:550-552 (hash & (n-1))
//
// The reference walks each run sequentially. Here every k-mer start position
// is decided independently: a k-mer starts a "chain" when it is the first
// k-mer of its run or its minimizer differs from the previous k-mer's; inside
// a chain a forced split falls every L = hdr_max + 1 - k k-mers after the
// chain start (the cap of partition_hash.hpp:81 replayed from the chain
// start); a record ends at the next cut or at the end of the run.
#include <algorithm>

#include "tg_internal.cuh"

namespace tg {

// ---------------------------------------------------------------- packing
// 2-bit kache codes (A0 C1 G2 T3, src/partition_hash.hpp:68-70) of every byte,
// 16 bases per u32 MSB-first, and one validity bit per base (ACGTacgt). Array
// base index a = stream position + TG_PAD. Grid-stride: a thread takes 64
// bases (four packed words, two validity words) per step, four bytes at a time
// with byte-wise SIMD compares; one atomic per CTA for the ACGT count.
__device__ __forceinline__ void pack_word4(uint32_t x, uint32_t& code8, uint32_t& ok4) {
    const uint32_t u = x & 0xDFDFDFDFu;  // upper case
    const uint32_t ok = __vcmpeq4(u, 0x41414141u) | __vcmpeq4(u, 0x43434343u) | __vcmpeq4(u, 0x47474747u) |
                        __vcmpeq4(u, 0x54545454u);
    // code ((c >> 2) ^ (c >> 1)) & 3 per byte, 0 where the byte is not ACGT
    const uint32_t t = (((x >> 2) ^ (x >> 1)) & 0x03030303u) & ok;
    // byte i's code to bits 6-2i of the result (first base most significant)
    code8 = (t * 0x40100401u) >> 24;
    ok4 = ((ok & 0x01010101u) * 0x01020408u) >> 24;
}

__global__ void __launch_bounds__(256) k_pack(const uint8_t* __restrict__ seq, uint64_t n,
                                              uint32_t* __restrict__ packed, uint32_t* __restrict__ valid,
                                              uint64_t n_groups, unsigned long long* __restrict__ n_bases) {
    __shared__ unsigned s_cnt;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    unsigned cnt = 0;
    const bool aligned = (reinterpret_cast<uintptr_t>(seq) & 15u) == 0;
    for (uint64_t gi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gi < n_groups;
         gi += (uint64_t)gridDim.x * blockDim.x) {
        const int64_t g0 = (int64_t)(gi * 64) - TG_PAD;
        uint32_t x[16];
        if (aligned && g0 >= 0 && (uint64_t)g0 + 64 <= n) {
            const uint4* p = reinterpret_cast<const uint4*>(seq + g0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 v = __ldcs(p + q);
                x[4 * q] = v.x;
                x[4 * q + 1] = v.y;
                x[4 * q + 2] = v.z;
                x[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int q = 0; q < 16; ++q) x[q] = 0;
#pragma unroll
            for (int i = 0; i < 64; ++i) {
                const int64_t g = g0 + i;
                if (g >= 0 && (uint64_t)g < n) x[i >> 2] |= (uint32_t)seq[g] << (8 * (i & 3));
            }
        }
        uint32_t pw[4], vw[2] = {0, 0};
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            uint32_t word = 0, vb = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t c8, o4;
                pack_word4(x[4 * w + q], c8, o4);
                word |= c8 << (24 - 8 * q);
                vb |= o4 << (4 * q);
            }
            pw[w] = word;
            vw[w >> 1] |= vb << (16 * (w & 1));
        }
        *reinterpret_cast<uint4*>(packed + 4 * gi) = make_uint4(pw[0], pw[1], pw[2], pw[3]);
        *reinterpret_cast<uint2*>(valid + 2 * gi) = make_uint2(vw[0], vw[1]);
        cnt += __popc(vw[0]) + __popc(vw[1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&s_cnt, cnt);
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt) atomicAdd(n_bases, (unsigned long long)s_cnt);
}

// ---------------------------------------------------------------- block scans
template <int NT>
struct BlockScan {
    // exclusive prefix sum of v over the block; returns it and the block total
    __device__ static uint32_t excl_sum(uint32_t v, uint32_t* s_warp, uint32_t& total) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            uint32_t t = lane < NT / 32 ? s_warp[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            if (lane < NT / 32) s_warp[lane] = t;
        }
        __syncthreads();
        total = s_warp[NT / 32 - 1];
        const uint32_t before = wid ? s_warp[wid - 1] : 0;
        __syncthreads();
        return before + x - v;
    }
    // exclusive prefix max of v (int64, -1 = none)
    __device__ static int64_t excl_max(int64_t v, int64_t* s_warp) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int64_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = max(x, y);
        }
        int64_t ex = __shfl_up_sync(0xffffffffu, x, 1);
        if (lane == 0) ex = -1;
        if (lane == 31) s_warp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int64_t t = lane < NT / 32 ? s_warp[lane] : -1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t = max(t, y);
            }
            if (lane < NT / 32) s_warp[lane] = t;
        }
        __syncthreads();
        const int64_t before = wid ? s_warp[wid - 1] : -1;
        __syncthreads();
        return max(before, ex);
    }
};

// Shared-memory layout of k_cut, sized at launch from w and the bucket count.
struct CutSmem {
    size_t tables, hist_r, hist_k, h, a, b, ev, evm, pk, vb, scan, total;
    int hn;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ void layout(int w, uint32_t p1, bool exp) {
        hn = CUT_TILE + w + 2;
        size_t o = 0;
        tables = o; o = align16(o + sizeof(HashTables));
        hist_r = o; o = align16(o + 4 * (size_t)p1);
        hist_k = o; o = align16(o + 4 * (size_t)p1);
        h = o; o = align16(o + 8 * (size_t)hn);
        a = o; o = align16(o + 8 * (size_t)hn);
        b = o; o = align16(o + 8 * (size_t)hn);
        ev = o; o = align16(o + 8 * (size_t)(CUT_TILE + 1));
        evm = o; o = align16(o + (exp ? 16 * (size_t)(CUT_TILE + 1) : 0));
        pk = o; o = align16(o + 4 * (size_t)(CUT_TILE + 2 * MAX_W + 320) / 16 + 64);
        vb = o; o = align16(o + 4 * (size_t)(CUT_TILE + 2 * MAX_W + 320) / 32 + 64);
        scan = o; o = align16(o + 8 * 64);
        total = o;
    }
};

// Exact min_pos of the reference's two-stack window (minimizer_window.hpp:
// 192-225, 317-325) for the k-mer whose m-mers are hashes hw[0..w]; q_off =
// (position of its last m-mer - run start) mod (w+1). Blocks of w+1 m-mers
// are aligned to the run start; the older block's minimum keeps its rightmost
// position on ties, the newer block's its leftmost, and a tie between the two
// goes to the newer block. When the k-mer's window is exactly one block
// (q_off == w) the rightmost minimum wins.
__device__ int ref_min_pos(const uint64_t* hw, int w, int q_off) {
    if (q_off == w) {
        uint64_t best = hw[0];
        int bp = 0;
        for (int j = 1; j <= w; ++j)
            if (hw[j] <= best) { best = hw[j]; bp = j; }
        return bp;
    }
    const int b0 = w - q_off;  // first index of the newer block
    uint64_t mo = ~0ull;
    int po = -1;
    for (int j = 0; j < b0; ++j)
        if (hw[j] <= mo) { mo = hw[j]; po = j; }
    uint64_t mn = hw[b0];
    int pn = b0;
    for (int j = b0 + 1; j <= w; ++j)
        if (hw[j] < mn) { mn = hw[j]; pn = j; }
    return (po >= 0 && mo < mn) ? po : pn;
}

// ---------------------------------------------------------------- superkmer cut
// One CTA per chunk of CTA-chunk k-mer start positions, walked in tiles of
// CUT_TILE. A CTA owns the chains that start inside its chunk and follows
// them past the chunk end until they close.
template <bool EXPORT>
__global__ void __launch_bounds__(CUT_THREADS, 2)
k_cut(CutParams P, const HashTables* __restrict__ gT) {
    extern __shared__ __align__(16) uint8_t smem[];
    CutSmem L;
    L.layout(P.w, 1u << P.p1_bits, EXPORT);
    HashTables& T = *reinterpret_cast<HashTables*>(smem + L.tables);
    uint32_t* s_hr = reinterpret_cast<uint32_t*>(smem + L.hist_r);
    uint32_t* s_hk = reinterpret_cast<uint32_t*>(smem + L.hist_k);
    uint64_t* s_h = reinterpret_cast<uint64_t*>(smem + L.h);
    uint64_t* s_a = reinterpret_cast<uint64_t*>(smem + L.a);
    uint64_t* s_b = reinterpret_cast<uint64_t*>(smem + L.b);
    uint2* s_ev = reinterpret_cast<uint2*>(smem + L.ev);
    uint64_t* s_evm = reinterpret_cast<uint64_t*>(smem + L.evm);  // EXPORT: hash, min_pos
    uint32_t* s_pk = reinterpret_cast<uint32_t*>(smem + L.pk);
    uint32_t* s_vb = reinterpret_cast<uint32_t*>(smem + L.vb);
    int64_t* s_scan64 = reinterpret_cast<int64_t*>(smem + L.scan);
    uint32_t* s_scan32 = reinterpret_cast<uint32_t*>(smem + L.scan + 8 * 32);
    __shared__ int64_t s_cs_carry;       // last chain start before the tile (-1: none)
    __shared__ int64_t s_open;           // start of the open owned record (-1: none)
    __shared__ uint32_t s_open_mlo;
    __shared__ uint64_t s_open_hash;
    __shared__ uint32_t s_open_mp;
    __shared__ uint32_t s_ndesc;
    __shared__ uint32_t s_nev;

    const int tid = threadIdx.x;
    const uint32_t p1 = 1u << P.p1_bits;
    const int k = P.k, m = P.m, w = P.w;
    const uint32_t c = blockIdx.x;
    {
        const uint64_t* src = reinterpret_cast<const uint64_t*>(gT);
        uint64_t* dst = reinterpret_cast<uint64_t*>(&T);
        for (int i = tid; i < (int)(sizeof(HashTables) / 8); i += CUT_THREADS) dst[i] = src[i];
        for (uint32_t i = tid; i < p1; i += CUT_THREADS) { s_hr[i] = 0; s_hk[i] = 0; }
        if (tid == 0) { s_cs_carry = -1; s_open = -1; s_ndesc = 0; }
    }
    __syncthreads();

    const uint64_t cstart = (uint64_t)c * P.chunk;
    const uint64_t cend = min(cstart + P.chunk, P.n);
    const int hn = L.hn;
    int plog = 0;
    while ((2 << plog) <= w + 1) ++plog;  // 2^plog <= w+1 < 2^(plog+1)
    const int pw = 1 << plog;
    uint64_t kmask_valid = (k >= 64) ? ~0ull : ((1ull << k) - 1);
    unsigned long long loc_kmers = 0, loc_recs = 0, loc_runs = 0;
    bool overflowed = false;

    for (uint64_t t0 = cstart; t0 < P.n; t0 += CUT_TILE) {
        if (t0 >= cend && s_open < 0) break;  // nothing of ours is still open
        // ---- stage packed and validity words: array bases [A0, A0 + NB)
        const uint64_t A0 = (t0 + TG_PAD - 1) & ~uint64_t(31);
        const int npk = (CUT_TILE + 2 * MAX_W + 320) / 16;
        for (int i = tid; i < npk; i += CUT_THREADS) s_pk[i] = P.packed[(A0 >> 4) + i];
        for (int i = tid; i < npk / 2; i += CUT_THREADS) s_vb[i] = P.valid[(A0 >> 5) + i];
        __syncthreads();
        // relative array index of global position g: g + TG_PAD - A0
        const uint64_t rel0 = TG_PAD - A0;  // add to g (mod 2^64)

        // ---- 1. canonical ntHash of m-mers q in [t0-1, t0+T+w]: index i = q - (t0-1)
        {
            constexpr int SEG = 8;
            for (int s0 = tid * SEG; s0 < hn; s0 += CUT_THREADS * SEG) {
                const uint64_t a = (t0 - 1) + (uint64_t)s0 + rel0;  // relative array index
                uint64_t f, r;
                nt_init(T, s_pk, a, m, f, r);
                s_h[s0] = f ^ r;
                const int e = min(SEG, hn - s0);
                for (int j = 1; j < e; ++j) {
                    const uint32_t out = base_at(s_pk, a + j - 1);
                    const uint32_t in = base_at(s_pk, a + j - 1 + m);
                    nt_roll(T, out, in, f, r);
                    s_h[s0 + j] = f ^ r;
                }
            }
        }
        __syncthreads();

        // ---- 2. minimizer of k-mers s in [t0-1, t0+T): M[i] = min h[i .. i+w]
        const uint64_t* Mv;
        {
            const uint64_t* src = s_h;
            uint64_t* bufs[2] = {s_a, s_b};
            for (int j = 1; j <= plog; ++j) {
                const int half = 1 << (j - 1);
                const int cnt = hn - ((1 << j) - 1);
                uint64_t* dst = bufs[(j - 1) & 1];
                for (int i = tid; i < cnt; i += CUT_THREADS) dst[i] = min(src[i], src[i + half]);
                __syncthreads();
                src = dst;
            }
            uint64_t* mdst = (src == s_a) ? s_b : s_a;
            const int off = w + 1 - pw;
            for (int i = tid; i <= CUT_TILE; i += CUT_THREADS) mdst[i] = min(src[i], src[i + off]);
            __syncthreads();
            Mv = mdst;
        }

        // ---- 3. flags of this thread's PT positions
        constexpr int PT = CUT_TILE / CUT_THREADS;
        bool vk[PT + 1];
        bool csf[PT], rs[PT], ev[PT];
        const uint64_t sbase = t0 + (uint64_t)tid * PT;
#pragma unroll
        for (int i = 0; i <= PT; ++i) {
            const uint64_t s = sbase + i - 1;  // i = 0 is the position before
            const uint64_t a = s + rel0;
            const uint64_t bits = valid64(s_vb, a);
            vk[i] = (s + 1 > 0) && s < P.n && ((~bits & kmask_valid) == 0);
            if (s == ~0ull) vk[i] = false;
        }
        int64_t last_cs = -1;
#pragma unroll
        for (int i = 0; i < PT; ++i) {
            const uint64_t s = sbase + i;
            const bool v = vk[i + 1];
            const bool prev_base = valid_base(s_vb, s - 1 + rel0);
            const bool first = v && !prev_base;
            const int mi = (int)(s - (t0 - 1));
            const bool hc = v && !first && Mv[mi] != Mv[mi - 1];
            csf[i] = first || hc;
            rs[i] = !v && vk[i];  // first invalid k-mer after a run: run end
            if (csf[i]) last_cs = (int64_t)s;
            if (first) ++loc_runs;
        }
        // chain start in force at each position: scan max across the tile
        int64_t before = BlockScan<CUT_THREADS>::excl_max(last_cs, s_scan64);
        before = max(before, s_cs_carry);
        uint32_t nev_local = 0;
        uint32_t owned_mask = 0;
        int64_t cs = before;
#pragma unroll
        for (int i = 0; i < PT; ++i) {
            const uint64_t s = sbase + i;
            const bool v = vk[i + 1];
            if (csf[i]) cs = (int64_t)s;
            bool forced = false;
            if (v && !csf[i] && cs >= 0) {
                const uint64_t d = s - (uint64_t)cs;
                forced = (d >= P.L) && (d % P.L == 0);
            }
            const bool cut = v && (csf[i] || forced);
            const bool owned = cut && cs >= (int64_t)cstart && cs < (int64_t)cend;
            ev[i] = cut || rs[i];
            if (owned) owned_mask |= 1u << i;
            nev_local += ev[i] ? 1u : 0u;
        }
        uint32_t nev_total;
        uint32_t ev_off = BlockScan<CUT_THREADS>::excl_sum(nev_local, s_scan32, nev_total);
        // ---- 4. event list (position order)
#pragma unroll
        for (int i = 0; i < PT; ++i) {
            if (!ev[i]) continue;
            const uint64_t s = sbase + i;
            const int mi = (int)(s - (t0 - 1));
            const bool own = (owned_mask >> i) & 1u;
            const uint64_t mval = Mv[mi];
            s_ev[ev_off] = make_uint2(((uint32_t)(s - t0) << 2) | (own ? EV_OWNED : 0u) | EV_CUT,
                                      (uint32_t)(mval & 0xFFFFFFu));
            if (EXPORT) {
                int mp = 0;
                if (own) {
                    // run start: scan validity bits backwards (export only)
                    uint64_t rsx = s;
                    while (rsx > 0 && valid_base(P.valid, rsx - 1 + TG_PAD)) {
                        const uint64_t aa = rsx - 1 + TG_PAD;
                        const uint32_t word = P.valid[aa >> 5];
                        const uint32_t bit = (uint32_t)(aa & 31);
                        const uint32_t below = (bit == 31) ? word : (word & ((2u << bit) - 1));
                        if (below == ((bit == 31) ? 0xFFFFFFFFu : ((2u << bit) - 1))) {
                            rsx -= bit + 1;  // whole word prefix valid
                        } else {
                            --rsx;
                        }
                    }
                    const int q_off = (int)((s + w - rsx) % (uint64_t)(w + 1));
                    mp = ref_min_pos(&s_h[mi], w, q_off);
                }
                s_evm[2 * ev_off] = mval;
                s_evm[2 * ev_off + 1] = (uint64_t)mp;
            }
            ++ev_off;
        }
        if (tid == 0) s_nev = nev_total;
        __syncthreads();
        // ---- 5. close records: event e closes the record opened at event e-1
        const uint32_t nev = s_nev;
        for (uint32_t base = 0; base < (nev + CUT_THREADS - 1) / CUT_THREADS * CUT_THREADS; base += CUT_THREADS) {
            const uint32_t e = base + tid;
            bool emit = false;
            uint64_t st = 0, mh = 0;
            uint32_t mlo = 0, nk = 0, mp = 0;
            if (e < nev) {
                const uint64_t pos = t0 + (s_ev[e].x >> 2);
                if (e == 0) {
                    if (s_open >= 0) {
                        emit = true;
                        st = (uint64_t)s_open;
                        mlo = s_open_mlo;
                        if (EXPORT) { mh = s_open_hash; mp = s_open_mp; }
                    }
                } else if (s_ev[e - 1].x & EV_OWNED) {
                    emit = true;
                    st = t0 + (s_ev[e - 1].x >> 2);
                    mlo = s_ev[e - 1].y;
                    if (EXPORT) { mh = s_evm[2 * (e - 1)]; mp = (uint32_t)s_evm[2 * (e - 1) + 1]; }
                }
                nk = (uint32_t)(pos - st);
            }
            uint32_t ntot;
            const uint32_t di = BlockScan<CUT_THREADS>::excl_sum(emit ? 1u : 0u, s_scan32, ntot);
            if (emit) {
                const uint32_t idx = s_ndesc + di;
                if (idx < P.desc_cap) {
                    P.desc[(uint64_t)c * P.desc_cap + idx] = desc_pack(st, nk, mlo);
                    if (EXPORT) {
                        uint64_t* x = P.xdesc + ((uint64_t)c * P.desc_cap + idx) * 3;
                        x[0] = st;
                        x[1] = mh;
                        x[2] = ((uint64_t)mp << 32) | nk;
                    }
                } else {
                    overflowed = true;
                }
                const uint32_t b = mlo & (p1 - 1);
                atomicAdd(&s_hr[b], 1u);
                atomicAdd(&s_hk[b], nk);
                loc_kmers += nk;
                loc_recs += 1;
            }
            __syncthreads();
            if (tid == 0) s_ndesc += ntot;
            __syncthreads();
        }
        // ---- 6. carries to the next tile
        if (tid == 0) {
            if (nev > 0) {
                const uint2 le = s_ev[nev - 1];
                if (le.x & EV_OWNED) {
                    s_open = (int64_t)(t0 + (le.x >> 2));
                    s_open_mlo = le.y;
                    if (EXPORT) { s_open_hash = s_evm[2 * (nev - 1)]; s_open_mp = (uint32_t)s_evm[2 * (nev - 1) + 1]; }
                } else {
                    s_open = -1;
                }
            }
        }
        // the tile's last chain start (thread with the highest position wins)
        if (tid == CUT_THREADS - 1) s_cs_carry = max(s_cs_carry, cs);
        __syncthreads();
    }
    // ---- flush histograms and counters
    for (uint32_t i = tid; i < p1; i += CUT_THREADS) {
        P.hist[(uint64_t)i * P.n_cta + c] = s_hr[i];
        if (s_hk[i]) atomicAdd(reinterpret_cast<unsigned long long*>(P.hist + hist_kmers_offset(p1, P.n_cta)) + i,
                               (unsigned long long)s_hk[i]);
    }
    if (tid == 0) P.n_desc[c] = s_ndesc;
    if (overflowed) atomicExch(P.overflow, 1u);
    // block-reduce the counters
    for (int o = 16; o > 0; o >>= 1) {
        loc_kmers += __shfl_down_sync(0xffffffffu, loc_kmers, o);
        loc_recs += __shfl_down_sync(0xffffffffu, loc_recs, o);
        loc_runs += __shfl_down_sync(0xffffffffu, loc_runs, o);
    }
    if ((tid & 31) == 0) {
        if (loc_kmers) atomicAdd(&P.stats[0], loc_kmers);
        if (loc_recs) atomicAdd(&P.stats[1], loc_recs);
        if (loc_runs) atomicAdd(&P.stats[2], loc_runs);
    }
}

// ---------------------------------------------------------------- sequential cut
// The counting path's cut (no export): each thread walks SEG consecutive k-mer
// start positions in order, as the reference walks a run, with a rolling
// ntHash and a block minimum over the window of w+1 m-mer hashes (van Herk /
// Gil-Werman: blocks of w+1 m-mers aligned to the thread's first m-mer; the
// window minimum is min(suffix minimum of the previous block, prefix minimum
// of the current one); the two per-thread buffers sit in shared memory, entry
// q of thread t at q * NT + t). Records whose start and end fall in one
// thread's segment are written during the walk; two block scans per tile of
// NT * SEG positions then give each thread the chain in force at its first
// position (for the forced split every L k-mers) and the next cut after its
// last one, which close the records that cross segments. A record that is open
// at the tile's end is carried to the next tile.
// 128 positions per thread: a thread walks SEG + w m-mers for SEG k-mers, so
// longer segments spend less on the window's warm-up (k=31 m=23: 7.43 ->
// 7.12 ms for 0.93 Gbp; k=63 m=21 reads: 13.35 -> 11.86 ms against 64). The
// forced split period L = 256 - k stays above SEG for every k <= 63, so a
// segment holds at most one forced split.
constexpr int SEG = 128;
static_assert(SEG * 256 <= CUT_SPAN, "a cut tile must fit the packed arrays' slack");

constexpr size_t SEQ_TABLE_BYTES = offsetof(HashTables, GF);

struct SeqSmem {
    size_t tables, pk, vb, vh, sum, total;
    uint32_t npk, nvb;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ void layout(int w, int nt, int k) {
        // bases [t0 - 1, t0 + nt * SEG + k) from a 32-base boundary
        const uint32_t span = (uint32_t)nt * SEG + (uint32_t)k + 96;
        npk = span / 16 + 2;
        nvb = span / 32 + 2;
        size_t o = 0;
        // the roll terms only (FW, RV, CTF, CTR): each thread's one initial hash
        // reads the 4-base group terms from global memory
        tables = o; o = align16(o + SEQ_TABLE_BYTES);
        pk = o; o = align16(o + 4 * (size_t)npk);
        vb = o; o = align16(o + 4 * (size_t)nvb);
        // one block of w + 1 hashes per thread: the block being filled, and from
        // its end back to the current offset the previous block's suffix minima
        vh = o; o = align16(o + 8 * (size_t)(w + 1) * nt);
        sum = o; o = align16(o + 20 * (size_t)nt);  // i64 chain, i64 first cut, u32 chain mlo
        total = o;
    }
};

// Threads of the sequential cut for window w (the block buffer holds w + 1
// hashes per thread).
__host__ __device__ inline int seq_threads(int w) { return w <= 15 ? 256 : (w <= 31 ? 128 : 64); }

// Exclusive max over lower threads of v (-1: none); `all` = inclusive max of the block.
template <int NT>
__device__ __forceinline__ int seq_excl_max(int v, int* s_w, int& all) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = max(x, y);
    }
    int ex = __shfl_up_sync(0xffffffffu, x, 1);
    if (lane == 0) ex = -1;
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < NT / 32 ? s_w[lane] : -1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t = max(t, y);
        }
        if (lane < NT / 32) s_w[lane] = t;
    }
    __syncthreads();
    const int before = wid ? s_w[wid - 1] : -1;
    all = s_w[NT / 32 - 1];
    __syncthreads();
    return max(before, ex);
}

// Exclusive min over higher threads of v (NT: none); `all` = min of the block.
template <int NT>
__device__ __forceinline__ int seq_excl_min_rev(int v, int* s_w, int& all) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = NT / 32;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_down_sync(0xffffffffu, x, o);
        if (lane + o < 32) x = min(x, y);
    }
    int ex = __shfl_down_sync(0xffffffffu, x, 1);
    if (lane == 31) ex = NT;
    if (lane == 0) s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < NW ? s_w[lane] : NT;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_down_sync(0xffffffffu, t, o);
            if (lane + o < 32) t = min(t, y);
        }
        if (lane < NW) s_w[lane] = t;
    }
    __syncthreads();
    const int after = wid + 1 < NW ? s_w[wid + 1] : NT;
    all = s_w[0];
    __syncthreads();
    return min(after, ex);
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 3 : 2)
k_cut_seq(CutParams P, const HashTables* __restrict__ gT) {
    extern __shared__ __align__(16) uint8_t smem[];
    SeqSmem L;
    L.layout(P.w, NT, P.k);
    HashTables& T = *reinterpret_cast<HashTables*>(smem + L.tables);
    uint32_t* s_pk = reinterpret_cast<uint32_t*>(smem + L.pk);
    uint32_t* s_vb = reinterpret_cast<uint32_t*>(smem + L.vb);
    uint64_t* vH = reinterpret_cast<uint64_t*>(smem + L.vh);
    // the previous block's suffix minima share the buffer: at offset o a step
    // writes hash o and reads suffix minimum o + 1, which is overwritten only at
    // the next step (k=63 m=21: half the shared memory, more CTAs per SM)
    uint64_t* vS = vH;
    int64_t* s_cs = reinterpret_cast<int64_t*>(smem + L.sum);  // chain in force after the segment's last cut
    int64_t* s_fe = s_cs + NT;                                  // the segment's first cut (-1: none)
    uint32_t* s_cm = reinterpret_cast<uint32_t*>(s_fe + NT);    // mlo of s_cs
    __shared__ int s_w[NT / 32];
    __shared__ int64_t s_carry_cs;   // chain in force at the tile start (-1: none)
    __shared__ uint32_t s_carry_m;
    __shared__ int64_t s_open;       // record open at the tile start (-1: none)
    __shared__ uint32_t s_open_m;
    __shared__ int s_open_own;
    __shared__ uint32_t s_ndesc;

    const int tid = threadIdx.x, lane = tid & 31;
    const int k = P.k, m = P.m, w = P.w, B = w + 1;
    const uint32_t c = blockIdx.x;
    {
        const uint64_t* src = reinterpret_cast<const uint64_t*>(gT);
        uint64_t* dst = reinterpret_cast<uint64_t*>(&T);  // T.GF and T.GR are not staged
        for (int i = tid; i < (int)(SEQ_TABLE_BYTES / 8); i += NT) dst[i] = src[i];
        if (tid == 0) { s_carry_cs = -1; s_carry_m = 0; s_open = -1; s_open_m = 0; s_open_own = 0; s_ndesc = 0; }
    }
    __syncthreads();

    const int64_t cstart = (int64_t)c * (int64_t)P.chunk;
    const int64_t cend = min(cstart + (int64_t)P.chunk, (int64_t)P.n);
    const uint64_t kmask = (1ull << k) - 1;  // k <= 63
    const int64_t Lr = P.L;
    unsigned long long loc_kmers = 0, loc_recs = 0, loc_runs = 0;
    bool overflowed = false;
    uint64_t* dlist = P.desc + (uint64_t)c * P.desc_cap;
    auto owned = [&](int64_t cs) { return cs >= cstart && cs < cend; };
    // sample holding position pos: the last i with sample_start[i] <= pos
    auto sample_of = [&](int64_t pos) -> uint32_t {
        uint32_t lo = 0, hi = P.n_samples - 1;
        while (lo < hi) {
            const uint32_t md = (lo + hi + 1) >> 1;
            if ((int64_t)P.sample_start[md] <= pos) lo = md; else hi = md - 1;
        }
        return lo;
    };
    // the thread's current segment [seg_lo, seg_lo + SEG) and, if it lies in one
    // sample, that sample (else ~0: look each record up)
    int64_t seg_lo = 0;
    uint32_t seg_s = 0;
    auto put = [&](uint32_t idx, int64_t st, uint32_t nk, uint32_t mh) {
        const uint32_t smp = (seg_s != ~0u && st >= seg_lo && st < seg_lo + SEG) ? seg_s : sample_of(st);
        const uint32_t bin = P.sample_bin_base[smp] + (mh & ((1u << P.sample_bin_bits[smp]) - 1));
        if (idx < P.desc_cap) dlist[idx] = desc_pack((uint64_t)st, nk, bin);
        else overflowed = true;
        atomicAdd(&P.binhist[bin], nk);  // the key array's layout
        loc_kmers += nk;
        loc_recs += 1;
    };
    // all lanes call this together; lanes with e write one record each
    auto emit_warp = [&](bool e, int64_t st, uint32_t nk, uint32_t mlo) {
        const unsigned bal = __ballot_sync(0xffffffffu, e);
        if (!bal) return;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&s_ndesc, (uint32_t)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (e) put(base + __popc(bal & ((1u << lane) - 1)), st, nk, mlo);
    };

    for (int64_t t0 = cstart; t0 < (int64_t)P.n; t0 += (int64_t)NT * SEG) {
        if (t0 >= cend && !(s_open >= 0 && s_open_own)) break;  // nothing of ours is still open
        // ---- stage packed and validity words: array bases [A0, A0 + 16 npk)
        const uint64_t A0 = (uint64_t)(t0 + TG_PAD - 1) & ~uint64_t(31);
        for (uint32_t i = tid; i < L.npk; i += NT) s_pk[i] = P.packed[(A0 >> 4) + i];
        for (uint32_t i = tid; i < L.nvb; i += NT) s_vb[i] = P.valid[(A0 >> 5) + i];
        __syncthreads();

        // ---- pass 1: walk positions [ps, ps + SEG) (m-mers from ps - 1 on).
        // Positions inside the walk are relative to pb = ps - 1 (32-bit). The
        // segments start SEG bases apart, so every thread crosses a packed word
        // (16 bases) or validity word (32) at the same step: the bases come
        // from register copies of the words, shifted once per step.
        const int64_t ps = t0 + (int64_t)tid * SEG;
        const int64_t pb = ps - 1;  // m-mer 0; k-mer kp = i - w starts at pb + kp
        seg_lo = ps;
        {
            const uint32_t a = sample_of(ps), b = sample_of(ps + SEG - 1);
            seg_s = a == b ? a : ~0u;
        }
        const uint32_t ra = (uint32_t)((uint64_t)(pb + TG_PAD) - A0);  // staged index of base pb
        uint64_t f, r;
        nt_init(*gT, s_pk, ra, m, f, r);
        int il;  // last invalid base entered so far, relative to pb (-1: none)
        {
            const uint64_t inval = ~valid64(s_vb, ra) & kmask;  // bases pb .. pb + k - 1
            il = inval ? 63 - __clzll((long long)inval) : -1;
        }
        auto rel = [&](int64_t x) {  // x - pb clamped to [-1, 2^31 - 1]: comparisons with kp keep
            const int64_t d = x - pb;
            return (int)(d < -1 ? -1 : (d > 0x7FFFFFFF ? 0x7FFFFFFF : d));
        };
        const int ownlo = rel(cstart), ownhi = rel(cend);
        uint32_t oi = ra, ii = ra + (uint32_t)m;  // bases leaving / entering at the next step
        uint32_t ow = s_pk[oi >> 4] << (2 * (oi & 15));
        uint32_t iw = s_pk[ii >> 4] << (2 * (ii & 15));
        uint32_t vw = s_vb[ii >> 5] >> (ii & 31);
        uint64_t h = f ^ r, pmin = h, mprev = 0;
        vH[tid] = h;  // m-mer 0 opens block 0 (w >= 1: no k-mer ends here)
        bool vprev = false, last_is_cs = false, open = false;
        int first_ev = -1, last_ev = -1, last_cs = -1, rs = 0;
        uint32_t rm = 0, last_cs_m = 0;
        int o = 1;  // offset of the m-mer in its block
        for (int i = 1; i <= SEG + w; ++i) {
            const uint32_t bo = ow >> 30, bi = iw >> 30, vb = vw & 1u;  // vb: base pb + i + m - 1
            ow <<= 2;
            iw <<= 2;
            vw >>= 1;
            ++oi;
            ++ii;
            if ((oi & 15) == 0) ow = s_pk[oi >> 4];
            if ((ii & 15) == 0) iw = s_pk[ii >> 4];
            if ((ii & 31) == 0) vw = s_vb[ii >> 5];
            nt_roll(T, bo, bi, f, r);
            h = f ^ r;
            vH[o * NT + tid] = h;
            pmin = min(pmin, h);
            if (i >= w) {
                const int kp = i - w;  // the k-mer whose window ends at this m-mer
                const uint64_t M = o == B - 1 ? pmin : min(vS[(o + 1) * NT + tid], pmin);
                if (i > w && !vb) il = kp + k - 1;  // its last base is pb + i + m - 1
                const bool v = il < kp;
                if (i > w) {
                    const bool first = v && !vprev;
                    const bool cs = v && (first || M != mprev);
                    const bool cut = cs || (!v && vprev);  // a new chain, or the end of a run
                    if (first && kp >= ownlo && kp < ownhi) ++loc_runs;
                    const bool close = cut && open && rs >= ownlo && rs < ownhi;
                    emit_warp(close, pb + rs, (uint32_t)(kp - rs), rm);
                    if (cut) {
                        if (first_ev < 0) first_ev = kp;
                        last_ev = kp;
                        last_is_cs = cs;
                        open = cs;
                        if (cs) { rs = kp; rm = (uint32_t)(M & 0xFFFFFu); last_cs = kp; last_cs_m = rm; }
                    }
                }
                mprev = M;
                vprev = v;
            }
            if (o == B - 1) {
                // block end: its suffix minima, for the windows of the next block
                uint64_t sm = ~0ull;
                for (int q = B - 1; q >= 0; --q) {
                    sm = min(sm, vH[q * NT + tid]);
                    vS[q * NT + tid] = sm;
                }
                pmin = ~0ull;
                o = 0;
            } else {
                ++o;
            }
        }
        // ---- chain in force at the segment start: the last cut of a lower thread
        s_cs[tid] = last_is_cs ? pb + last_cs : -1;
        s_cm[tid] = last_cs_m;
        const int64_t first_abs = first_ev >= 0 ? pb + first_ev : -1;
        int last_t;
        const int prev = seq_excl_max<NT>(last_ev >= 0 ? tid : -1, s_w, last_t);
        int64_t cs_in = s_carry_cs;
        uint32_t m_in = s_carry_m;
        if (prev >= 0) { cs_in = s_cs[prev]; m_in = s_cm[prev]; }
        // forced split of that chain inside the segment (L > SEG: at most one)
        int64_t fc = -1;
        if (cs_in >= 0) {
            const int64_t d = ps - cs_in;
            const int64_t rem = d % Lr;
            const int64_t cand = ps + (rem ? Lr - rem : 0);
            if (cand < ps + SEG && (first_abs < 0 || cand < first_abs)) fc = cand;
        }
        // a forced-split record closed by the segment's first cut
        emit_warp(fc >= 0 && first_abs >= 0 && owned(cs_in), fc, (uint32_t)(first_abs - fc), m_in);
        // the record open at the segment's end, if it starts in the segment
        bool oo = false, oown = false;
        int64_t os = 0;
        uint32_t om = 0;
        if (open) { oo = true; os = pb + rs; om = rm; oown = owned(os); }
        else if (fc >= 0 && first_abs < 0) { oo = true; os = fc; om = m_in; oown = owned(cs_in); }
        const int64_t fe = fc >= 0 ? fc : first_abs;
        s_fe[tid] = fe;
        int first_t;
        const int nxt = seq_excl_min_rev<NT>(fe >= 0 ? tid : NT, s_w, first_t);
        emit_warp(oo && nxt < NT && oown, os, nxt < NT ? (uint32_t)(s_fe[nxt] - os) : 0u, om);
        // ---- tile carries: the record open at the tile start closes at the
        // tile's first cut; the last open record and the last chain carry on
        if (tid == 0 && first_t < NT && s_open >= 0) {
            if (s_open_own) put(atomicAdd(&s_ndesc, 1u), s_open, (uint32_t)(s_fe[first_t] - s_open), s_open_m);
            s_open = -1;
        }
        __syncthreads();
        if (oo && nxt == NT) { s_open = os; s_open_m = om; s_open_own = oown ? 1 : 0; }
        if (tid == 0 && last_t >= 0) { s_carry_cs = s_cs[last_t]; s_carry_m = s_cm[last_t]; }
        __syncthreads();
    }
    // ---- counters
    if (tid == 0) P.n_desc[c] = s_ndesc;
    if (overflowed) atomicExch(P.overflow, 1u);
    for (int o = 16; o > 0; o >>= 1) {
        loc_kmers += __shfl_down_sync(0xffffffffu, loc_kmers, o);
        loc_recs += __shfl_down_sync(0xffffffffu, loc_recs, o);
        loc_runs += __shfl_down_sync(0xffffffffu, loc_runs, o);
    }
    if (lane == 0) {
        if (loc_kmers) atomicAdd(&P.stats[0], loc_kmers);
        if (loc_recs) atomicAdd(&P.stats[1], loc_recs);
        if (loc_runs) atomicAdd(&P.stats[2], loc_runs);
    }
}

// ---------------------------------------------------------------- fixed-(k, m) cut
// The sequential cut compiled for one (k, m) with a window of B = k - m + 1 <= 16
// m-mers (the reference compiles one binary per (k, m) too, FIXED_K/FIXED_M).
// Same walk and the same records as k_cut_seq; what the fixed shape buys:
//  * the window minimum is a van Herk block minimum whose two arrays (the
//    current block's hashes, the previous block's suffix minima) are register
//    arrays: the loop is unrolled by whole blocks, so every index is static;
//  * the per-position work is only the roll, the window minimum and one bit
//    "minimizer changed" (plus the minimizer's low bits, kept in shared memory
//    for the chain starts). Validity, chain starts, run ends, forced-split
//    bookkeeping and record emission are done once per batch of R blocks
//    (R * B <= 32 k-mers) with bit operations on 32-bit masks: k-mer validity is
//    a run-AND of k validity bits, a chain starts at a valid k-mer that is the
//    first of its run or whose minimizer changed, a run ends at the first
//    invalid k-mer after a valid one;
//  * records that close inside the batch get their slots from one warp scan and
//    one shared atomic per warp and batch.
// The bases that leave and enter the m-mer during a batch come from two 64-bit
// windows of the staged packed words, read once per batch and shifted by one
// base per roll. The ntHash roll terms CTF/CTR are interleaved (one 16-byte
// shared load per base). Measured on 0.93 Gbp of the assembly (k=31 m=23, one
// GB300): 5.51 ms with per-roll base words, 5.18 with the per-batch windows,
// 5.11 with the segment's first bin cached as well (k_cut_seq: 7.1);
// 128-thread CTAs gave 5.59, 192 positions per thread 6.13. Everything after
// the walk (the scans across threads, the forced split every L k-mers, the
// records that cross segments, the tile carries) is the code of k_cut_seq.
template <int K, int MM>
struct FixedShape {
    static constexpr int W = K - MM, B = W + 1;
    static constexpr int R = 32 / B;            // blocks per batch
    static constexpr int SB = R * B;            // k-mers per batch (<= 32)
    static constexpr int NBLK = (SEG + B - 1) / B;
    static constexpr int NT = 256;
    static_assert(B >= 2 && B <= 16, "fixed cut: window of 2..16 m-mers");
};

// Shared-memory layout of k_cut_fixed.
struct FixedSmem {
    size_t tables, ct, pk, vb, mlo, sum, total;
    uint32_t npk, nvb;
    __host__ __device__ static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
    __host__ __device__ void layout(int nt, int k) {
        // bases [t0 - 1, t0 + nt * SEG + 16 + k) from a 32-base boundary, with
        // room for the validity window of the last batch (128 bits)
        const uint32_t span = (uint32_t)nt * SEG + (uint32_t)k + 288;
        npk = span / 16 + 2;
        nvb = span / 32 + 2;
        size_t o = 0;
        tables = o; o = align16(o + sizeof(HashTables));
        ct = o; o = align16(o + 16 * 16);
        pk = o; o = align16(o + 4 * (size_t)npk);
        vb = o; o = align16(o + 4 * (size_t)nvb);
        mlo = o; o = align16(o + 4 * 32 * (size_t)nt);
        sum = o; o = align16(o + 20 * (size_t)nt);
        total = o;
    }
};

// 128 bits of b starting at bit index a (bit 0 of the result = bit a).
__device__ __forceinline__ void bits128(const uint32_t* b, uint32_t a, uint64_t& lo, uint64_t& hi) {
    const uint32_t w = a >> 5, o = a & 31;
    const uint32_t x0 = b[w], x1 = b[w + 1], x2 = b[w + 2], x3 = b[w + 3], x4 = b[w + 4];
    const uint32_t y0 = o ? __funnelshift_r(x0, x1, o) : x0;
    const uint32_t y1 = o ? __funnelshift_r(x1, x2, o) : x1;
    const uint32_t y2 = o ? __funnelshift_r(x2, x3, o) : x2;
    const uint32_t y3 = o ? __funnelshift_r(x3, x4, o) : x3;
    lo = ((uint64_t)y1 << 32) | y0;
    hi = ((uint64_t)y3 << 32) | y2;
}

__device__ __forceinline__ void shr128(uint64_t lo, uint64_t hi, int s, uint64_t& rlo, uint64_t& rhi) {
    if (s == 0) { rlo = lo; rhi = hi; }
    else if (s < 64) { rlo = (lo >> s) | (hi << (64 - s)); rhi = hi >> s; }
    else { rlo = hi >> (s - 64); rhi = 0; }
}

// Bit j (j < 64) of the result: bits [j, j + K) of v are all set (K <= 64).
template <int K>
__device__ __forceinline__ uint64_t run_and(uint64_t lo, uint64_t hi) {
    uint64_t acc_lo = ~0ull, acc_hi = ~0ull;
    uint64_t cl = lo, ch = hi;  // runs of `len` set bits starting at each bit
    int off = 0;
#pragma unroll
    for (int b = 0; b < 7; ++b) {
        const int len = 1 << b;
        if (K & len) {
            uint64_t sl, sh;
            shr128(cl, ch, off, sl, sh);
            acc_lo &= sl;
            acc_hi &= sh;
            off += len;
        }
        if ((K >> (b + 1)) == 0) break;
        uint64_t sl, sh;
        shr128(cl, ch, len, sl, sh);
        cl &= sl;
        ch &= sh;
    }
    return acc_lo;
}

constexpr uint32_t FIXED_CUT_CTAS = 3;  // CTAs of 256 threads per SM

template <int K, int MM>
__global__ void __launch_bounds__(256, FIXED_CUT_CTAS)
k_cut_fixed(CutParams P, const HashTables* __restrict__ gT) {
    using S = FixedShape<K, MM>;
    constexpr int NT = S::NT, W = S::W, B = S::B, SB = S::SB, R = S::R;
    extern __shared__ __align__(16) uint8_t smem[];
    FixedSmem Ly;
    Ly.layout(NT, K);
    HashTables& T = *reinterpret_cast<HashTables*>(smem + Ly.tables);
    ulonglong2* s_ct = reinterpret_cast<ulonglong2*>(smem + Ly.ct);   // {CTF, CTR}[16]
    uint32_t* s_pk = reinterpret_cast<uint32_t*>(smem + Ly.pk);
    uint32_t* s_vb = reinterpret_cast<uint32_t*>(smem + Ly.vb);
    uint32_t* s_mlo = reinterpret_cast<uint32_t*>(smem + Ly.mlo);     // [SB][NT] minimizer low bits
    int64_t* s_cs = reinterpret_cast<int64_t*>(smem + Ly.sum);
    int64_t* s_fe = s_cs + NT;
    uint32_t* s_cm = reinterpret_cast<uint32_t*>(s_fe + NT);
    __shared__ int s_w[NT / 32];
    __shared__ int64_t s_carry_cs;
    __shared__ uint32_t s_carry_m;
    __shared__ int64_t s_open;
    __shared__ uint32_t s_open_m;
    __shared__ int s_open_own;
    __shared__ uint32_t s_ndesc;

    const int tid = threadIdx.x, lane = tid & 31;
    const uint32_t c = blockIdx.x;
    {
        const uint64_t* src = reinterpret_cast<const uint64_t*>(gT);
        uint64_t* dst = reinterpret_cast<uint64_t*>(&T);
        for (int i = tid; i < (int)(sizeof(HashTables) / 8); i += NT) dst[i] = src[i];
        if (tid < 16) s_ct[tid] = make_ulonglong2(gT->CTF[tid], gT->CTR[tid]);
        if (tid == 0) { s_carry_cs = -1; s_carry_m = 0; s_open = -1; s_open_m = 0; s_open_own = 0; s_ndesc = 0; }
    }
    __syncthreads();

    const int64_t cstart = (int64_t)c * (int64_t)P.chunk;
    const int64_t cend = min(cstart + (int64_t)P.chunk, (int64_t)P.n);
    const int64_t Lr = P.L;
    unsigned long long loc_kmers = 0, loc_recs = 0, loc_runs = 0;
    bool overflowed = false;
    uint64_t* dlist = P.desc + (uint64_t)c * P.desc_cap;
    auto owned = [&](int64_t cs) { return cs >= cstart && cs < cend; };
    auto sample_of = [&](int64_t pos) -> uint32_t {
        uint32_t lo = 0, hi = P.n_samples - 1;
        while (lo < hi) {
            const uint32_t md = (lo + hi + 1) >> 1;
            if ((int64_t)P.sample_start[md] <= pos) lo = md; else hi = md - 1;
        }
        return lo;
    };
    // the segment's sample when the segment lies in one (its first bin and bin
    // mask cached), else a lookup per record
    int64_t seg_lo = 0;
    uint32_t seg_s = 0, seg_base = 0, seg_mask = 0;
    auto put = [&](uint32_t idx, int64_t st, uint32_t nk, uint32_t mh) {
        uint32_t bin;
        if (seg_s != ~0u && st >= seg_lo && st < seg_lo + SEG) {
            bin = seg_base + (mh & seg_mask);
        } else {
            const uint32_t smp = sample_of(st);
            bin = P.sample_bin_base[smp] + (mh & ((1u << P.sample_bin_bits[smp]) - 1));
        }
        if (idx < P.desc_cap) dlist[idx] = desc_pack((uint64_t)st, nk, bin);
        else overflowed = true;
        atomicAdd(&P.binhist[bin], nk);
        loc_kmers += nk;
        loc_recs += 1;
    };
    auto emit_warp = [&](bool e, int64_t st, uint32_t nk, uint32_t mlo) {
        const unsigned bal = __ballot_sync(0xffffffffu, e);
        if (!bal) return;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&s_ndesc, (uint32_t)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (e) put(base + __popc(bal & ((1u << lane) - 1)), st, nk, mlo);
    };

    for (int64_t t0 = cstart; t0 < (int64_t)P.n; t0 += (int64_t)NT * SEG) {
        if (t0 >= cend && !(s_open >= 0 && s_open_own)) break;
        const uint64_t A0 = (uint64_t)(t0 + TG_PAD - 1) & ~uint64_t(31);
        for (uint32_t i = tid; i < Ly.npk; i += NT) s_pk[i] = P.packed[(A0 >> 4) + i];
        for (uint32_t i = tid; i < Ly.nvb; i += NT) s_vb[i] = P.valid[(A0 >> 5) + i];
        __syncthreads();

        const int64_t ps = t0 + (int64_t)tid * SEG;
        const int64_t pb = ps - 1;
        seg_lo = ps;
        {
            const uint32_t a = sample_of(ps), b = sample_of(ps + SEG - 1);
            seg_s = a == b ? a : ~0u;
            seg_base = P.sample_bin_base[a];
            seg_mask = (1u << P.sample_bin_bits[a]) - 1;
        }
        const uint32_t ra = (uint32_t)((uint64_t)(pb + TG_PAD) - A0);  // staged index of base pb
        auto rel = [&](int64_t x) {
            const int64_t d = x - pb;
            return (int)(d < -1 ? -1 : (d > 0x7FFFFFFF ? 0x7FFFFFFF : d));
        };
        const int ownlo = rel(cstart), ownhi = rel(cend);
        // ---- warm-up: m-mers 0 .. B-1 (block 0); k-mer 0 ends at m-mer W
        uint64_t f, r;
        nt_init(T, s_pk, ra, MM, f, r);
        uint64_t cur[B], sfx[B];
        // the bases leaving and entering the m-mer, 32 at a time: 64-bit windows
        // of the staged packed words (the roll into m-mer i takes out base
        // pb + i - 1 and in base pb + i - 1 + MM), shifted by one base per roll
        uint64_t wob = window64(s_pk, ra), wib = window64(s_pk, ra + MM);
        auto roll = [&]() -> uint64_t {
            const uint32_t bo = (uint32_t)(wob >> 62), bi = (uint32_t)(wib >> 62);
            wob <<= 2;
            wib <<= 2;
            const ulonglong2 t = s_ct[(bo << 2) | bi];
            f = ((f << 1) | (f >> 63)) ^ t.x;
            r = ((r >> 1) | (r << 63)) ^ t.y;
            return f ^ r;
        };
        cur[0] = f ^ r;
        uint64_t pmin = cur[0];
#pragma unroll
        for (int o = 1; o < B; ++o) {
            cur[o] = roll();
            pmin = min(pmin, cur[o]);
        }
#pragma unroll
        for (int q = B - 1; q >= 0; --q) sfx[q] = q == B - 1 ? cur[q] : min(cur[q], sfx[q + 1]);
        uint64_t mprev = pmin;  // minimizer of k-mer 0
        // ---- state of the walk
        bool open = false, last_is_cs = false;
        int first_ev = -1, last_ev = -1, last_cs = -1, rs = 0;
        uint32_t rm = 0, last_cs_m = 0;
        // ---- batches of R blocks (SB k-mers): k-mers kp0 .. kp0 + SB - 1
        for (int kp0 = 1; kp0 <= SEG; kp0 += SB) {
            uint32_t chg = 0;
            {  // the batch's m-mers kp0 + W + j roll out base pb + kp0 + W - 1 + j
                const uint32_t a0 = ra + (uint32_t)(kp0 + W - 1);
                wob = window64(s_pk, a0);
                wib = window64(s_pk, a0 + MM);
            }
#pragma unroll
            for (int rb = 0; rb < R; ++rb) {
                if (kp0 + rb * B > SEG) break;  // the segment's last blocks (uniform)
#pragma unroll
                for (int o = 0; o < B; ++o) {
                    const uint64_t h = roll();
                    cur[o] = h;
                    pmin = o == 0 ? h : min(pmin, h);
                    const uint64_t M = o == B - 1 ? pmin : min(sfx[o + 1], pmin);
                    const int j = rb * B + o;
                    chg |= (M != mprev ? 1u : 0u) << j;
                    s_mlo[j * NT + tid] = (uint32_t)M;
                    mprev = M;
                }
#pragma unroll
                for (int q = B - 1; q >= 0; --q) sfx[q] = q == B - 1 ? cur[q] : min(cur[q], sfx[q + 1]);
            }
            // k-mers of this batch inside the segment: bits [0, nb)
            const int nb = min(SB, SEG + 1 - kp0);
            const uint32_t inseg = nb >= 32 ? ~0u : ((1u << nb) - 1);
            // validity of k-mers kp0 - 1 .. kp0 + 31: run-AND of K validity bits
            uint64_t vlo, vhi;
            bits128(s_vb, ra + (uint32_t)(kp0 - 1), vlo, vhi);
            const uint64_t vr = run_and<K>(vlo, vhi);
            const uint32_t vk = (uint32_t)(vr >> 1) & inseg;   // bit j: k-mer kp0 + j valid
            const uint32_t vpm = (vk << 1) | (uint32_t)(vr & 1u);  // bit j: k-mer kp0 + j - 1 valid
            const uint32_t first = vk & ~vpm;
            const uint32_t cs = vk & (first | chg);
            const uint32_t cut = (cs | (~vk & vpm)) & inseg;
            // own range of this batch: bits j with ownlo <= kp0 + j < ownhi
            const int olo = min(max(ownlo - kp0, 0), 32), ohi = min(max(ownhi - kp0, 0), 32);
            const uint32_t own = (uint32_t)(((olo >= 32 ? 0ull : (~0ull << olo)) & ((1ull << ohi) - 1)));
            loc_runs += __popc(first & own);
            // records closed inside the batch: the open record at the first cut,
            // and every owned chain start followed by another cut
            uint32_t nrec = 0, top = 0, cl = 0;
            if (cut) {
                top = 31 - __clz(cut);
                cl = cs & own & ~(1u << top);
                nrec = __popc(cl) + ((open && rs >= ownlo && rs < ownhi) ? 1u : 0u);
            }
            uint32_t incl = nrec;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += y;
            }
            const uint32_t wtot = __shfl_sync(0xffffffffu, incl, 31);
            if (wtot) {
                uint32_t base = 0;
                if (lane == 31) base = atomicAdd(&s_ndesc, wtot);
                base = __shfl_sync(0xffffffffu, base, 31);
                uint32_t idx = base + incl - nrec;
                if (cut) {
                    const int f0 = __ffs(cut) - 1;
                    if (open && rs >= ownlo && rs < ownhi) put(idx++, pb + rs, (uint32_t)(kp0 + f0 - rs), rm);
                    while (cl) {
                        const int cb = __ffs(cl) - 1;
                        cl &= cl - 1;
                        const uint32_t after = cut & (uint32_t)(~0ull << (cb + 1));
                        const int e = __ffs(after) - 1;
                        put(idx++, pb + kp0 + cb, (uint32_t)(e - cb), s_mlo[cb * NT + tid] & 0xFFFFFu);
                    }
                }
            }
            if (cut) {
                if (first_ev < 0) first_ev = kp0 + __ffs(cut) - 1;
                last_ev = kp0 + (int)top;
                last_is_cs = (cs >> top) & 1u;
                if (cs) {
                    const int lc = 31 - __clz(cs);
                    last_cs = kp0 + lc;
                    last_cs_m = s_mlo[lc * NT + tid] & 0xFFFFFu;
                }
                open = last_is_cs;
                if (open) { rs = last_cs; rm = last_cs_m; }
            }
        }
        // ---- as k_cut_seq: chain in force at the segment start, forced split,
        // records crossing segments, tile carries
        s_cs[tid] = last_is_cs ? pb + last_cs : -1;
        s_cm[tid] = last_cs_m;
        const int64_t first_abs = first_ev >= 0 ? pb + first_ev : -1;
        int last_t;
        const int prev = seq_excl_max<NT>(last_ev >= 0 ? tid : -1, s_w, last_t);
        int64_t cs_in = s_carry_cs;
        uint32_t m_in = s_carry_m;
        if (prev >= 0) { cs_in = s_cs[prev]; m_in = s_cm[prev]; }
        int64_t fc = -1;
        if (cs_in >= 0) {
            const int64_t d = ps - cs_in;
            const int64_t rem = d % Lr;
            const int64_t cand = ps + (rem ? Lr - rem : 0);
            if (cand < ps + SEG && (first_abs < 0 || cand < first_abs)) fc = cand;
        }
        emit_warp(fc >= 0 && first_abs >= 0 && owned(cs_in), fc, (uint32_t)(first_abs - fc), m_in);
        bool oo = false, oown = false;
        int64_t os = 0;
        uint32_t om = 0;
        if (open) { oo = true; os = pb + rs; om = rm; oown = owned(os); }
        else if (fc >= 0 && first_abs < 0) { oo = true; os = fc; om = m_in; oown = owned(cs_in); }
        const int64_t fe = fc >= 0 ? fc : first_abs;
        s_fe[tid] = fe;
        int first_t;
        const int nxt = seq_excl_min_rev<NT>(fe >= 0 ? tid : NT, s_w, first_t);
        emit_warp(oo && nxt < NT && oown, os, nxt < NT ? (uint32_t)(s_fe[nxt] - os) : 0u, om);
        if (tid == 0 && first_t < NT && s_open >= 0) {
            if (s_open_own) put(atomicAdd(&s_ndesc, 1u), s_open, (uint32_t)(s_fe[first_t] - s_open), s_open_m);
            s_open = -1;
        }
        __syncthreads();
        if (oo && nxt == NT) { s_open = os; s_open_m = om; s_open_own = oown ? 1 : 0; }
        if (tid == 0 && last_t >= 0) { s_carry_cs = s_cs[last_t]; s_carry_m = s_cm[last_t]; }
        __syncthreads();
    }
    if (tid == 0) P.n_desc[c] = s_ndesc;
    if (overflowed) atomicExch(P.overflow, 1u);
    for (int o = 16; o > 0; o >>= 1) {
        loc_kmers += __shfl_down_sync(0xffffffffu, loc_kmers, o);
        loc_recs += __shfl_down_sync(0xffffffffu, loc_recs, o);
        loc_runs += __shfl_down_sync(0xffffffffu, loc_runs, o);
    }
    if (lane == 0) {
        if (loc_kmers) atomicAdd(&P.stats[0], loc_kmers);
        if (loc_recs) atomicAdd(&P.stats[1], loc_recs);
        if (loc_runs) atomicAdd(&P.stats[2], loc_runs);
    }
}

// ---------------------------------------------------------------- offsets
// Exclusive scan of two u32 arrays of length n into u64 outputs, one CTA per
// SCAN_ITEMS items, then a fix-up with the scanned block sums.
constexpr int SCAN_T = 1024, SCAN_ITEMS = 8192;

__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint64_t n, unsigned long long* __restrict__ out,
                              unsigned long long* __restrict__ block_sums) {
    __shared__ unsigned long long s[SCAN_T];
    const uint64_t b0 = (uint64_t)blockIdx.x * SCAN_ITEMS;
    constexpr int PER = SCAN_ITEMS / SCAN_T;
    unsigned long long v[PER], acc = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const uint64_t idx = b0 + (uint64_t)threadIdx.x * PER + i;
        v[i] = idx < n ? in[idx] : 0;
        acc += v[i];
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 1; o < SCAN_T; o <<= 1) {
        const unsigned long long y = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += y;
        __syncthreads();
    }
    unsigned long long run = s[threadIdx.x] - acc;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const uint64_t idx = b0 + (uint64_t)threadIdx.x * PER + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
    if (threadIdx.x == SCAN_T - 1) block_sums[blockIdx.x] = s[SCAN_T - 1];
}

__global__ void k_scan_sums(unsigned long long* __restrict__ sums, uint32_t nb, unsigned long long* __restrict__ total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long acc = 0;
        for (uint32_t i = 0; i < nb; ++i) {
            const unsigned long long v = sums[i];
            sums[i] = acc;
            acc += v;
        }
        *total = acc;
    }
}

__global__ void k_scan_add(unsigned long long* __restrict__ out, uint64_t n, const unsigned long long* __restrict__ sums) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / SCAN_ITEMS];
}

// ---------------------------------------------------------------- launchers
// (k, m) pairs with a compiled cut (k_cut_fixed): the bench and served
// workloads' shapes; other pairs take k_cut_seq.
static bool fixed_cut(int k, int w) {
    const int m = k - w;
    return (k == 31 && (m == 21 || m == 23)) || (k == 21 && m == 17) || (k == 25 && m == 21);
}

size_t cut_smem_bytes(int w, int k, uint32_t p1, bool exp) {
    if (exp) {
        CutSmem L;
        L.layout(w, p1, exp);
        return L.total;
    }
    if (fixed_cut(k, w)) {
        FixedSmem F;
        F.layout(256, k);
        return F.total;
    }
    SeqSmem L;
    L.layout(w, seq_threads(w), k);
    return L.total;
}

uint64_t cut_tile(int w, bool exp) { return exp ? (uint64_t)CUT_TILE : (uint64_t)seq_threads(w) * SEG; }

uint32_t cut_ctas_per_sm(int w, int k, uint32_t p1, bool exp) {
    const size_t sm = cut_smem_bytes(w, k, p1, exp) + 1024;
    const uint32_t by_smem = (uint32_t)(228u * 1024u / sm);
    if (!exp && fixed_cut(k, w)) return std::max<uint32_t>(1, std::min<uint32_t>(FIXED_CUT_CTAS, by_smem));
    // the sequential cut: up to 768 threads per SM (three CTAs of 256; for wide
    // windows, 64-thread CTAs as many as shared memory allows: k=63 m=21 reads,
    // 3 -> 4 CTAs, 11.9 -> 9.0 ms for 0.9 Gbp; one block buffer instead of two,
    // 4 -> 7 CTAs)
    return std::max<uint32_t>(1, std::min<uint32_t>(exp ? 2u : 768u / (uint32_t)seq_threads(w), by_smem));
}

cudaError_t launch_pack(const uint8_t* seq, uint64_t n, uint32_t* packed, uint32_t* valid, uint64_t n_words,
                        unsigned long long* n_bases, cudaStream_t st) {
    // n_words is a multiple of 4 (packed_words_for): groups of 4 words
    const uint64_t groups = n_words / 4;
    int dev = 0, n_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t threads = 256;
    const uint64_t blocks = std::min<uint64_t>((groups + threads - 1) / threads, (uint64_t)std::max(n_sm, 1) * 8);
    k_pack<<<(unsigned)std::max<uint64_t>(blocks, 1), threads, 0, st>>>(seq, n, packed, valid, groups, n_bases);
    return cudaGetLastError();
}

uint64_t packed_words_for(uint64_t n) {
    const uint64_t pw = (TG_PAD + n + CUT_SPAN + 2 * MAX_W + 640) / 16 + 16;
    return (pw + 3) & ~uint64_t(3);
}

template <int NT>
static cudaError_t launch_cut_seq(const CutParams& P, const HashTables* gT, size_t sm, cudaStream_t st) {
    const cudaError_t e = set_smem_cap(k_cut_seq<NT>, sm);
    if (e != cudaSuccess) return e;
    k_cut_seq<NT><<<P.n_cta, NT, sm, st>>>(P, gT);
    return cudaGetLastError();
}

template <int K, int MM>
static cudaError_t launch_cut_fixed(const CutParams& P, const HashTables* gT, size_t sm, cudaStream_t st) {
    const cudaError_t e = set_smem_cap(k_cut_fixed<K, MM>, sm);
    if (e != cudaSuccess) return e;
    k_cut_fixed<K, MM><<<P.n_cta, FixedShape<K, MM>::NT, sm, st>>>(P, gT);
    return cudaGetLastError();
}

cudaError_t launch_cut(const CutParams& P, const HashTables* gT, bool exp, cudaStream_t st) {
    const size_t sm = cut_smem_bytes(P.w, P.k, 1u << P.p1_bits, exp);
    if (!exp && fixed_cut(P.k, P.w)) {
        switch (P.k * 100 + P.m) {
            case 3121: return launch_cut_fixed<31, 21>(P, gT, sm, st);
            case 3123: return launch_cut_fixed<31, 23>(P, gT, sm, st);
            case 2117: return launch_cut_fixed<21, 17>(P, gT, sm, st);
            default: return launch_cut_fixed<25, 21>(P, gT, sm, st);
        }
    }
    if (exp) {
        const cudaError_t e = set_smem_cap(k_cut<true>, sm);
        if (e != cudaSuccess) return e;
        k_cut<true><<<P.n_cta, CUT_THREADS, sm, st>>>(P, gT);
        return cudaGetLastError();
    }
    switch (seq_threads(P.w)) {
        case 256: return launch_cut_seq<256>(P, gT, sm, st);
        case 128: return launch_cut_seq<128>(P, gT, sm, st);
        default: return launch_cut_seq<64>(P, gT, sm, st);
    }
}

cudaError_t launch_scan(const uint32_t* in, uint64_t n, unsigned long long* out, unsigned long long* sums,
                        unsigned long long* total, cudaStream_t st, int* launches) {
    const uint32_t nb = (uint32_t)((n + SCAN_ITEMS - 1) / SCAN_ITEMS);
    k_scan_blocks<<<nb, SCAN_T, 0, st>>>(in, n, out, sums);
    k_scan_sums<<<1, 32, 0, st>>>(sums, nb, total);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, sums);
    *launches += 3;
    return cudaGetLastError();
}


}  // namespace tg
