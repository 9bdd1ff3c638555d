// tg_lex.cu — FASTA/FASTQ lexing on the device: the raw bytes of one input
// file in, the sequence stream the counting kernels take out (the ACGT runs
// the reference's parser hands to extract_superkmers_from_actg, separated by
// non-ACGT bytes).
//
// Rules (the host parser in host/fastx.cpp states them at length):
//  * FASTA (include/helicase_cpp/parser_fasta.hpp:233-316): bytes before the
//    first '>' are ignored; '>' (anywhere in a sequence line) starts a header
//    that runs to the next LF; in sequence, LF bytes are dropped (lines join)
//    and every other byte is kept (non-ACGT bytes then separate runs). Each
//    header start is written as one separator byte.
//  * FASTQ (include/helicase_cpp/parser_fastq.hpp:112-285): line i of the
//    file is a sequence line iff i = 1 (mod 4); sequence lines are kept with
//    their LF. The reference walks the file in 64-byte blocks, which differs
//    from plain line counting in two places only:
//      - an empty header line whose LF is the last byte of a 64-byte block
//        (file offset 63 mod 64) is merged with the following line. The lexer
//        flags such files (LexTotals::irregular) and the caller parses them on
//        the host instead;
//      - when the file length is a multiple of 64 and the file ends inside a
//        sequence line on an ACGT byte, the run reaching the end is dropped.
//
// Three kernels, no inter-CTA waits. Each CTA owns a contiguous range of
// 16 KiB chunks, which TMA bulk copies stage into shared memory (two buffers);
// each thread owns one 64-byte block of a chunk (file offsets 64t..64t+63),
// made into bit masks (LF, '>', ACGT) with byte-wise SIMD compares.
//  k_lex_sum   the summary of the lexer automaton over the CTA's range for
//              each start state (end state, bytes emitted);
//  k_lex_scan  one CTA: the state and output offset at the start of each range;
//  k_lex_emit  each range again from its start: bytes emitted through shared
//              memory and written with 16-byte stores.
#include "tg_launch.h"

namespace tg {
namespace {

constexpr int LEX_THREADS = 256;
constexpr uint64_t LEX_CHUNK = (uint64_t)LEX_THREADS * 64;  // bytes per CTA step

// Summary of a byte range for each of the 4 start states s: end state
// (2 bits at 2s of e) and the number of bytes emitted.
template <typename C>
struct LexFn {
    uint32_t e;
    C c0, c1, c2, c3;
};

template <typename C>
__device__ __forceinline__ LexFn<C> lex_identity() {
    return LexFn<C>{0xE4u, 0, 0, 0, 0};
}
__device__ __forceinline__ uint32_t lex_end(uint32_t e, uint32_t s) { return (e >> (2 * s)) & 3u; }
template <typename C>
__device__ __forceinline__ C lex_cnt(const LexFn<C>& f, uint32_t s) {
    return s == 0 ? f.c0 : s == 1 ? f.c1 : s == 2 ? f.c2 : f.c3;
}
// a, then b
template <typename C>
__device__ __forceinline__ LexFn<C> lex_then(const LexFn<C>& a, const LexFn<C>& b) {
    const uint32_t m0 = a.e & 3u, m1 = (a.e >> 2) & 3u, m2 = (a.e >> 4) & 3u, m3 = (a.e >> 6) & 3u;
    LexFn<C> r;
    r.e = lex_end(b.e, m0) | (lex_end(b.e, m1) << 2) | (lex_end(b.e, m2) << 4) | (lex_end(b.e, m3) << 6);
    r.c0 = a.c0 + lex_cnt(b, m0);
    r.c1 = a.c1 + lex_cnt(b, m1);
    r.c2 = a.c2 + lex_cnt(b, m2);
    r.c3 = a.c3 + lex_cnt(b, m3);
    return r;
}
template <typename C>
__device__ __forceinline__ LexFn<C> lex_shfl_down(const LexFn<C>& f, int d) {
    return LexFn<C>{__shfl_down_sync(~0u, f.e, d), __shfl_down_sync(~0u, f.c0, d), __shfl_down_sync(~0u, f.c1, d),
                    __shfl_down_sync(~0u, f.c2, d), __shfl_down_sync(~0u, f.c3, d)};
}
template <typename C>
__device__ __forceinline__ LexFn<C> lex_shfl_up(const LexFn<C>& f, int d) {
    return LexFn<C>{__shfl_up_sync(~0u, f.e, d), __shfl_up_sync(~0u, f.c0, d), __shfl_up_sync(~0u, f.c1, d),
                    __shfl_up_sync(~0u, f.c2, d), __shfl_up_sync(~0u, f.c3, d)};
}
// inclusive ordered scan over the lanes of a warp
template <typename C>
__device__ __forceinline__ LexFn<C> lex_warp_scan(LexFn<C> f, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const LexFn<C> o = lex_shfl_up(f, d);
        if (lane >= d) f = lex_then(o, f);
    }
    return f;
}

// One 64-byte block as 16 little-endian words (byte i in bits 8(i%4) of word
// i/4) and the mask of bytes inside the file.
__device__ __forceinline__ void lex_load(const uint8_t* __restrict__ raw, uint64_t len, uint64_t base,
                                         uint32_t (&w)[16], uint64_t& valid) {
    if (base + 64 <= len) {
        const uint4* p = reinterpret_cast<const uint4*>(raw + base);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 v = __ldcs(p + q);
            w[4 * q] = v.x;
            w[4 * q + 1] = v.y;
            w[4 * q + 2] = v.z;
            w[4 * q + 3] = v.w;
        }
        valid = ~0ull;
        return;
    }
    const uint64_t nv = base < len ? len - base : 0;  // < 64
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = 0;
#pragma unroll
    for (int i = 0; i < 64; ++i)
        if ((uint64_t)i < nv) w[i >> 2] |= (uint32_t)raw[base + i] << (8 * (i & 3));
    valid = nv ? (~0ull >> (64 - nv)) : 0ull;
}

// bit j of the result = byte j of the word is 0xFF in m (a __vcmpeq4 result)
__device__ __forceinline__ uint32_t lex_nib(uint32_t m) { return ((m & 0x01010101u) * 0x01020408u) >> 24; }

__device__ __forceinline__ uint64_t lex_eq_mask(const uint32_t (&w)[16], uint32_t pat) {
    uint64_t r = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) r |= (uint64_t)lex_nib(__vcmpeq4(w[q], pat)) << (4 * q);
    return r;
}
__device__ __forceinline__ uint64_t lex_acgt_mask(const uint32_t (&w)[16]) {
    uint64_t r = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const uint32_t u = w[q] & 0xDFDFDFDFu;  // upper case
        const uint32_t a = __vcmpeq4(u, 0x41414141u) | __vcmpeq4(u, 0x43434343u) | __vcmpeq4(u, 0x47474747u) |
                           __vcmpeq4(u, 0x54545454u);
        r |= (uint64_t)lex_nib(a) << (4 * q);
    }
    return r;
}

// FASTA automaton over the bytes in rem from state s: 0 before the first '>',
// 1 in a header, 2 in sequence. emit receives the bytes written.
__device__ __forceinline__ uint32_t fa_walk(uint64_t gt, uint64_t lf, uint64_t rem, uint32_t s, uint64_t& emit) {
    emit = 0;
    for (int it = 0; it < 130 && rem; ++it) {  // every step consumes one set bit of rem or stops
        if (s == 1) {
            const uint64_t l = lf & rem;
            if (!l) break;
            const uint64_t b = l & (0ull - l);
            rem &= ~(b | (b - 1));
            s = 2;
        } else {
            const uint64_t g = gt & rem;
            const uint64_t b = g & (0ull - g);
            if (s == 2) emit |= (g ? (rem & (b - 1)) : rem) & ~lf;
            if (!g) break;
            emit |= b;
            rem &= ~(b | (b - 1));
            s = 1;
        }
    }
    return s;
}

// FASTQ: the bytes of the block by line index relative to the block start
// mod 4 (a line's LF belongs to it): R[r] = bytes on lines r, r+4, ...
__device__ __forceinline__ void fq_lines(uint64_t lf, uint64_t rem, uint64_t& R0, uint64_t& R1, uint64_t& R2,
                                         uint64_t& R3) {
    R0 = R1 = R2 = R3 = 0;
    uint32_t j = 0;
    for (int it = 0; it < 66 && rem; ++it) {
        const uint64_t l = lf & rem;
        const uint64_t b = l & (0ull - l);
        const uint64_t seg = l ? (rem & ((b << 1) - 1)) : rem;
        const uint32_t r = j & 3u;
        R0 |= r == 0 ? seg : 0;
        R1 |= r == 1 ? seg : 0;
        R2 |= r == 2 ? seg : 0;
        R3 |= r == 3 ? seg : 0;
        rem &= ~seg;
        ++j;
    }
}
// bytes emitted from line state s (line index at the block start mod 4)
__device__ __forceinline__ uint64_t fq_emit(uint64_t R0, uint64_t R1, uint64_t R2, uint64_t R3, uint32_t s) {
    return s == 0 ? R1 : s == 1 ? R0 : s == 2 ? R3 : R2;
}

// ---- TMA staging: whole 16 KiB chunks are copied into shared memory by one
// bulk copy (cp.async.bulk) completing on an mbarrier; every wait is bounded
// (1 s of the global timer) and a timeout is reported, never waited out.
constexpr uint64_t WAIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void tma_chunk(void* dst, const void* src, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"((uint32_t)LEX_CHUNK)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"((uint32_t)LEX_CHUNK), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint64_t t0 = gtimer();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (gtimer() - t0 > WAIT_NS) return false;
    }
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// A CTA's chunks: a contiguous range, whole chunks double-buffered through
// shared memory (buffer it & 1 for the it-th chunk of the range); the file's
// last, partial chunk is read from global memory directly.
struct LexStage {
    uint8_t (*buf)[LEX_CHUNK + 32];
    uint64_t* bar;
    const uint8_t* raw;
    uint64_t len, c_lo, c_hi, n_full;

    __device__ __forceinline__ void issue(uint64_t c, uint32_t it) const {
        if (c < c_hi && c < n_full) tma_chunk(buf[it & 1], raw + c * LEX_CHUNK, &bar[it & 1]);
    }
    // this thread's 64 bytes of chunk c (the it-th of the range); false on a timeout
    __device__ __forceinline__ bool get(uint64_t c, uint32_t it, uint32_t (&w)[16], uint64_t& valid) const {
        if (c < n_full) {
            const bool ok = mbar_wait(&bar[it & 1], (it >> 1) & 1);
            if (__syncthreads_or(!ok)) return false;
            const uint4* p = reinterpret_cast<const uint4*>(buf[it & 1] + threadIdx.x * 64);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 v = p[q];
                w[4 * q] = v.x;
                w[4 * q + 1] = v.y;
                w[4 * q + 2] = v.z;
                w[4 * q + 3] = v.w;
            }
            valid = ~0ull;
        } else {
            lex_load(raw, len, c * LEX_CHUNK + threadIdx.x * 64, w, valid);
        }
        return true;
    }
    // after a timeout: wait (bounded) for the copies this CTA still has in flight
    __device__ __forceinline__ void drain(uint64_t c, uint32_t it) const {
        if (threadIdx.x != 0) return;
        if (c < n_full) mbar_wait(&bar[it & 1], (it >> 1) & 1);
        if (c + 1 < c_hi && c + 1 < n_full) mbar_wait(&bar[(it + 1) & 1], ((it + 1) >> 1) & 1);
    }
};

template <int FASTQ>
struct LexBlock {
    uint32_t w[16];
    uint64_t valid, lf, gt, R0, R1, R2, R3;
    LexFn<uint32_t> f;

    __device__ __forceinline__ void build() {
        lf = lex_eq_mask(w, 0x0A0A0A0Au) & valid;
        if (!FASTQ) {
            gt = lex_eq_mask(w, 0x3E3E3E3Eu) & valid;
            uint64_t em;
            const uint32_t e0 = fa_walk(gt, lf, valid, 0, em);
            f.c0 = __popcll(em);
            const uint32_t e1 = fa_walk(gt, lf, valid, 1, em);
            f.c1 = __popcll(em);
            const uint32_t e2 = fa_walk(gt, lf, valid, 2, em);
            f.c2 = __popcll(em);
            f.c3 = 0;
            f.e = e0 | (e1 << 2) | (e2 << 4) | (3u << 6);
        } else {
            fq_lines(lf, valid, R0, R1, R2, R3);
            const uint32_t nl = __popcll(lf);
            f.c0 = __popcll(R1);
            f.c1 = __popcll(R0);
            f.c2 = __popcll(R3);
            f.c3 = __popcll(R2);
            f.e = (nl & 3u) | (((1u + nl) & 3u) << 2) | (((2u + nl) & 3u) << 4) | (((3u + nl) & 3u) << 6);
        }
    }
};

constexpr int LEX_CTAS_PER_SM = 3;
constexpr uint32_t LEX_MAX_CTAS = 4096;
typedef unsigned long long ull;

// Pass 1: the summary of each CTA's range of chunks.
template <int FASTQ>
__global__ void __launch_bounds__(LEX_THREADS, LEX_CTAS_PER_SM)
    k_lex_sum(const uint8_t* __restrict__ raw, uint64_t len, uint64_t n_chunks, uint64_t per_cta,
              LexFn<ull>* __restrict__ fn, long long* __restrict__ last_na, LexTotals* tot) {
    __shared__ __align__(128) uint8_t s_in[2][LEX_CHUNK + 32];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ LexFn<uint32_t> s_w[LEX_THREADS / 32];
    __shared__ long long s_na;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LexStage S{s_in, s_bar, raw, len, 0, 0, len / LEX_CHUNK};
    S.c_lo = min(n_chunks, (uint64_t)blockIdx.x * per_cta);
    S.c_hi = min(n_chunks, S.c_lo + per_cta);
    if (threadIdx.x == 0) {
        mbar_init(&s_bar[0]);
        mbar_init(&s_bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_na = -1;
    }
    __syncthreads();
    if (threadIdx.x == 0) S.issue(S.c_lo, 0);
    LexFn<ull> carry = lex_identity<ull>();
    uint32_t it = 0;
    for (uint64_t c = S.c_lo; c < S.c_hi; ++c, ++it) {
        if (threadIdx.x == 0) S.issue(c + 1, it + 1);
        LexBlock<FASTQ> B;
        if (!S.get(c, it, B.w, B.valid)) {
            if (threadIdx.x == 0) atomicOr(&tot->irregular, 2u);
            S.drain(c, it);
            return;
        }
        B.build();
        LexFn<uint32_t> f = B.f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const LexFn<uint32_t> o = lex_shfl_down(f, d);
            if ((lane & (2 * d - 1)) == 0) f = lex_then(f, o);
        }
        if (lane == 0) s_w[warp] = f;
        if (FASTQ) {  // last non-ACGT byte (for the end-of-file rule)
            const uint64_t na = ~lex_acgt_mask(B.w) & B.valid;
            if (na) atomicMax(&s_na, (long long)(c * LEX_CHUNK + threadIdx.x * 64 + 63 - __clzll(na)));
        }
        __syncthreads();
        if (warp == 0) {  // the warps' summaries in order, by a shuffle tree over lanes 0..7
            LexFn<uint32_t> g = lane < LEX_THREADS / 32 ? s_w[lane] : lex_identity<uint32_t>();
#pragma unroll
            for (int d = 1; d < LEX_THREADS / 32; d <<= 1) {
                const LexFn<uint32_t> o = lex_shfl_down(g, d);
                if ((lane & (2 * d - 1)) == 0) g = lex_then(g, o);
            }
            if (lane == 0) carry = lex_then(carry, LexFn<ull>{g.e, g.c0, g.c1, g.c2, g.c3});
        }
        fence_proxy_async();  // this buffer's reads before the next bulk copy into it
        __syncthreads();      // buffer it & 1 and s_w free for reuse
    }
    if (threadIdx.x == 0) {
        fn[blockIdx.x] = carry;
        if (FASTQ) last_na[blockIdx.x] = s_na;
    }
}

constexpr int SCAN_THREADS = 1024;

template <typename C>
__device__ __forceinline__ LexFn<C> lex_bcast(const LexFn<C>& f, int src) {
    return LexFn<C>{__shfl_sync(~0u, f.e, src), __shfl_sync(~0u, f.c0, src), __shfl_sync(~0u, f.c1, src),
                    __shfl_sync(~0u, f.c2, src), __shfl_sync(~0u, f.c3, src)};
}

// Pass 2, one CTA: the state and output offset at the start of each range.
// Warp w reads a contiguous run of the range summaries 32 at a time.
__global__ void __launch_bounds__(SCAN_THREADS) k_lex_scan(const LexFn<ull>* __restrict__ fn, uint64_t n_items,
                                                           int fastq, uint64_t len, const long long* __restrict__ last_na,
                                                           uint8_t* __restrict__ cstate, ull* __restrict__ coff,
                                                           LexTotals* tot) {
    constexpr int NW = SCAN_THREADS / 32;
    __shared__ LexFn<ull> s_w[NW];
    __shared__ ull s_off[NW];
    __shared__ uint32_t s_st[NW];
    __shared__ long long s_na;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_na = -1;
    __syncthreads();
    const uint64_t per = (n_items + NW - 1) / NW;
    const uint64_t lo = min(n_items, (uint64_t)warp * per), hi = min(n_items, lo + per);
    LexFn<ull> agg = lex_identity<ull>();
    long long na = -1;
    for (uint64_t b = lo; b < hi; b += 32) {
        const uint64_t c = b + lane;
        LexFn<ull> g = c < hi ? fn[c] : lex_identity<ull>();
        if (fastq && c < hi) na = max(na, last_na[c]);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const LexFn<ull> o = lex_shfl_down(g, d);
            if ((lane & (2 * d - 1)) == 0) g = lex_then(g, o);
        }
        agg = lex_then(agg, lex_bcast(g, 0));
    }
    if (fastq) {
#pragma unroll
        for (int d = 16; d; d >>= 1) na = max(na, (long long)__shfl_xor_sync(~0u, (ull)na, d));
        if (lane == 0 && na >= 0) atomicMax(&s_na, na);
    }
    if (lane == 0) s_w[warp] = agg;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        ull off = 0;
        for (int i = 0; i < NW; ++i) {
            s_st[i] = s;
            s_off[i] = off;
            off += lex_cnt(s_w[i], s);
            s = lex_end(s_w[i].e, s);
        }
        ull drop = len;
        // FASTQ, length a multiple of 64, file ending on an ACGT byte of a
        // sequence line: the run reaching the end is dropped
        const long long lna = s_na;
        if (fastq && s == 1 && len && (len & 63) == 0 && lna < (long long)len - 1) {
            drop = (ull)(lna + 1);
            off -= len - drop;
        }
        tot->out = off;
        tot->drop_from = drop;
        tot->final_state = s;
    }
    __syncthreads();
    uint32_t s = s_st[warp];
    ull off = s_off[warp];
    for (uint64_t b = lo; b < hi; b += 32) {
        const uint64_t c = b + lane;
        const LexFn<ull> g = c < hi ? fn[c] : lex_identity<ull>();
        const LexFn<ull> incl = lex_warp_scan(g, lane);
        LexFn<ull> ex = lex_shfl_up(incl, 1);
        if (lane == 0) ex = lex_identity<ull>();
        if (c < hi) {
            cstate[c] = (uint8_t)lex_end(ex.e, s);
            coff[c] = off + lex_cnt(ex, s);
        }
        const LexFn<ull> last = lex_bcast(incl, 31);
        off += lex_cnt(last, s);
        s = lex_end(last.e, s);
    }
}

// Pass 3: each CTA walks its range again from its start state and offset and
// writes the stream. Per chunk: the threads' summaries scanned within each
// warp, the warps chained from the chunk's start state by one thread, the
// emitted bytes staged in the chunk's (now read) shared buffer, then written
// with 16-byte stores.
template <int FASTQ>
__global__ void __launch_bounds__(LEX_THREADS, LEX_CTAS_PER_SM)
    k_lex_emit(const uint8_t* __restrict__ raw, uint64_t len, uint64_t n_chunks, uint64_t per_cta,
               const uint8_t* __restrict__ cstate, const ull* __restrict__ coff, LexTotals* tot,
               uint8_t* __restrict__ out) {
    __shared__ __align__(128) uint8_t s_in[2][LEX_CHUNK + 32];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ LexFn<uint32_t> s_wf[LEX_THREADS / 32];
    __shared__ uint32_t s_ws[LEX_THREADS / 32], s_wo[LEX_THREADS / 32];
    __shared__ uint32_t s_state, s_cnt;
    __shared__ ull s_off;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LexStage S{s_in, s_bar, raw, len, 0, 0, len / LEX_CHUNK};
    S.c_lo = min(n_chunks, (uint64_t)blockIdx.x * per_cta);
    S.c_hi = min(n_chunks, S.c_lo + per_cta);
    const ull total = tot->out, drop = tot->drop_from;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar[0]);
        mbar_init(&s_bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (S.c_lo < S.c_hi) {
            s_state = cstate[blockIdx.x];
            s_off = coff[blockIdx.x];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) S.issue(S.c_lo, 0);
    uint32_t it = 0;
    for (uint64_t c = S.c_lo; c < S.c_hi; ++c, ++it) {
        if (threadIdx.x == 0) S.issue(c + 1, it + 1);
        LexBlock<FASTQ> B;
        if (!S.get(c, it, B.w, B.valid)) {
            if (threadIdx.x == 0) atomicOr(&tot->irregular, 2u);
            S.drain(c, it);
            return;
        }
        B.build();
        const LexFn<uint32_t> incl = lex_warp_scan(B.f, lane);
        if (lane == 31) s_wf[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t st = s_state, o = 0;
#pragma unroll
            for (int i = 0; i < LEX_THREADS / 32; ++i) {
                s_ws[i] = st;
                s_wo[i] = o;
                o += lex_cnt(s_wf[i], st);
                st = lex_end(s_wf[i].e, st);
            }
            s_cnt = o;
            s_state = st;  // the next chunk's start state (read only after the next barrier)
        }
        __syncthreads();
        LexFn<uint32_t> ex = lex_shfl_up(incl, 1);
        if (lane == 0) ex = lex_identity<uint32_t>();
        const uint32_t ws = s_ws[warp];
        const uint32_t s = lex_end(ex.e, ws);
        const uint32_t o = s_wo[warp] + lex_cnt(ex, ws);
        const uint64_t base = c * LEX_CHUNK + threadIdx.x * 64;
        uint64_t em;
        if (!FASTQ) {
            fa_walk(B.gt, B.lf, B.valid, s, em);
        } else {
            em = fq_emit(B.R0, B.R1, B.R2, B.R3, s);
            if (base + 64 > drop) em &= drop > base ? (~0ull >> (64 - (drop - base))) : 0ull;
            // empty header line ending at file offset 63 mod 64
            if ((B.lf >> 62) == 3ull && ((s + __popcll(B.lf & (~0ull >> 1))) & 3u) == 0)
                atomicOr(&tot->irregular, 1u);
        }
        const ull g0 = s_off;
        const uint32_t chunk_cnt = s_cnt;
        uint8_t* stage = s_in[it & 1];  // every thread has its bytes in registers
        const uint32_t sh = (uint32_t)(((uintptr_t)out + g0) & 15u);
        uint32_t p = sh + o;
#pragma unroll
        for (int i = 0; i < 64; ++i) {
            if ((em >> i) & 1ull) {
                uint32_t b = (B.w[i >> 2] >> (8 * (i & 3))) & 0xFFu;
                if (!FASTQ && b == '>') b = '\n';
                stage[p++] = (uint8_t)b;
            }
        }
        __syncthreads();
        const ull end = min(g0 + chunk_cnt, total);
        if (end > g0) {
            const long long a0 = (long long)g0 - (long long)sh;  // out + a0 is 16-byte aligned
            const uint32_t n16 = (uint32_t)((end - a0 + 15) / 16);
            for (uint32_t u = threadIdx.x; u < n16; u += LEX_THREADS) {
                const long long ga = a0 + 16ll * u;
                if (ga >= (long long)g0 && ga + 16 <= (long long)end) {
                    *reinterpret_cast<uint4*>(out + ga) = *reinterpret_cast<const uint4*>(stage + 16 * u);
                } else {
                    for (int b = 0; b < 16; ++b) {
                        const long long g = ga + b;
                        if (g >= (long long)g0 && g < (long long)end) out[g] = stage[16 * u + b];
                    }
                }
            }
        }
        fence_proxy_async();  // generic accesses to this buffer before the next bulk copy into it
        __syncthreads();
        if (threadIdx.x == 0) s_off = g0 + chunk_cnt;
    }
}

}  // namespace

size_t lex_scratch_bytes(uint64_t len) {
    (void)len;
    return 256 + 4 * 256 + (size_t)LEX_MAX_CTAS * (sizeof(LexFn<ull>) + 8 + 8 + 1);
}

cudaError_t launch_lex(const uint8_t* raw, uint64_t len, bool fastq, uint8_t* out, void* scratch, int n_sm,
                       cudaStream_t st, LexTotals** dtot, int* launches) {
    const uint64_t nc = (len + LEX_CHUNK - 1) / LEX_CHUNK;
    const uint64_t G = std::max<uint64_t>(1, std::min<uint64_t>({nc, (uint64_t)n_sm * LEX_CTAS_PER_SM, LEX_MAX_CTAS}));
    const uint64_t per = (nc + G - 1) / std::max<uint64_t>(G, 1);
    uint8_t* p = static_cast<uint8_t*>(scratch);
    auto take = [&](size_t bytes) {
        uint8_t* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    LexTotals* tot = reinterpret_cast<LexTotals*>(take(sizeof(LexTotals)));
    LexFn<ull>* fn = reinterpret_cast<LexFn<ull>*>(take(G * sizeof(LexFn<ull>)));
    long long* last_na = reinterpret_cast<long long*>(take(G * 8));
    ull* coff = reinterpret_cast<ull*>(take(G * 8));
    uint8_t* cstate = take(G);
    *dtot = tot;
    cudaError_t e = cudaMemsetAsync(tot, 0, sizeof(LexTotals), st);
    if (e != cudaSuccess || nc == 0) return e;
    if (fastq) k_lex_sum<1><<<(unsigned)G, LEX_THREADS, 0, st>>>(raw, len, nc, per, fn, last_na, tot);
    else k_lex_sum<0><<<(unsigned)G, LEX_THREADS, 0, st>>>(raw, len, nc, per, fn, last_na, tot);
    k_lex_scan<<<1, SCAN_THREADS, 0, st>>>(fn, G, fastq ? 1 : 0, len, last_na, cstate, coff, tot);
    if (fastq) k_lex_emit<1><<<(unsigned)G, LEX_THREADS, 0, st>>>(raw, len, nc, per, cstate, coff, tot, out);
    else k_lex_emit<0><<<(unsigned)G, LEX_THREADS, 0, st>>>(raw, len, nc, per, cstate, coff, tot, out);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

}  // namespace tg
