/*
 * tuna_oracle.c — CPU restatement of the reference tuna counting path.
 *
 * TEST INFRASTRUCTURE, NOT THE PRODUCT: what the GPU library's results are
 * compared with, and the CPU baseline that bench.py times. See tuna_oracle.h for the map from each
 * stage to the reference file it follows. The restatement is pinned against the
 * reference's own binaries (oracle/build_ref.sh) and the fixtures they produced
 * (tests/golden/).
 */
#define _GNU_SOURCE
#include "tuna_oracle.h"
#include "tuna_digest.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Byte classes (include/helicase_cpp/simd.hpp:299-343, scalar lexer).      */
/* A byte is DNA iff (x & 0xDF) == "A_C_T_G_"[x & 6]: exactly [ACGTacgt].   */

static inline int is_acgt(uint8_t x) {
    static const uint8_t lut[8] = {'A', 0, 'C', 0, 'T', 0, 'G', 0};
    return (uint8_t)(x & 0xDFu) == lut[x & 6u];
}

/* ------------------------------------------------------------------------ */
/* Growable byte buffer                                                      */

typedef struct {
    uint8_t* p;
    size_t n, cap;
} bbuf;

static void bb_reserve(bbuf* b, size_t need) {
    if (need <= b->cap) return;
    size_t c = b->cap ? b->cap : 256;
    while (c < need) c *= 2;
    uint8_t* q = (uint8_t*)realloc(b->p, c);
    if (!q) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    b->p = q;
    b->cap = c;
}
static inline void bb_put(bbuf* b, const uint8_t* s, size_t n) {
    bb_reserve(b, b->n + n);
    memcpy(b->p + b->n, s, n);
    b->n += n;
}
static inline uint8_t* bb_grow(bbuf* b, size_t n) {
    bb_reserve(b, b->n + n);
    uint8_t* r = b->p + b->n;
    b->n += n;
    return r;
}
static void bb_free(bbuf* b) { free(b->p); b->p = NULL; b->n = b->cap = 0; }

/* ------------------------------------------------------------------------ */
/* FASTA (parser_fasta.hpp:233-316 with the lexer masks of lexer.hpp:46-68). */
/* Byte-level form of the same state machine: everything before the first   */
/* '>' is skipped; a header runs from '>' through the next LF; inside        */
/* sequence LF bytes are transparent, ACGT bytes extend the run, and any     */
/* other byte (N, '\r', '>' which opens a header, ...) ends the run.         */

static void fasta_runs(const uint8_t* d, size_t n, tor_run_cb cb, void* user) {
    enum { BEFORE, HEADER, SEQ } st = BEFORE;
    bbuf run = {0};
    for (size_t i = 0; i < n; ++i) {
        const uint8_t c = d[i];
        switch (st) {
        case BEFORE:
            if (c == '>') st = HEADER;
            break;
        case HEADER:
            if (c == '\n') st = SEQ;
            break;
        case SEQ:
            if (is_acgt(c)) {
                /* extend: copy the maximal ACGT stretch at once */
                size_t j = i;
                while (j < n && is_acgt(d[j])) ++j;
                bb_put(&run, d + i, j - i);
                i = j - 1;
            } else if (c == '\n') {
                /* transparent */
            } else {
                if (run.n) { cb(run.p, run.n, user); run.n = 0; }
                if (c == '>') st = HEADER;
            }
            break;
        }
    }
    if (st == SEQ && run.n) cb(run.p, run.n, user);
    bb_free(&run);
}

/* ------------------------------------------------------------------------ */
/* FASTQ (parser_fastq.hpp:112-285). The reference walks 64-byte blocks and  */
/* keeps, per block, the mask of newlines not yet consumed; a record is four */
/* lines and only line 2 is scanned. The block structure is kept here       */
/* because it decides the behaviour on malformed input (blank lines, a      */
/* final line with no LF).                                                   */

typedef struct {
    const uint8_t* d;
    size_t n;
    size_t blk;      /* index of the current block */
    size_t blen;     /* bytes of the current block */
    size_t pos;      /* position inside the block */
    uint64_t nl;     /* unconsumed newline bits */
    uint64_t dna;    /* DNA bits (ACGT, not LF) */
    int finished;
    int line;
} fq_state;

static void fq_load(fq_state* s, size_t b) {
    const size_t off = b * 64;
    s->blk = b;
    s->blen = (s->n - off) < 64 ? (s->n - off) : 64;
    s->pos = 0;
    uint64_t nl = 0, dna = 0;
    for (size_t i = 0; i < 64; ++i) {
        const uint8_t x = i < s->blen ? s->d[off + i] : 0;
        if (x == '\n') nl |= 1ull << i;
        if (is_acgt(x)) dna |= 1ull << i;
    }
    s->nl = nl;
    s->dna = dna & ~nl;
}
/* returns 1 at end of input */
static int fq_advance(fq_state* s) {
    const size_t nb = s->blk + 1;
    if (nb * 64 >= s->n) { s->finished = 1; return 1; }
    fq_load(s, nb);
    return 0;
}
static void fq_incr(fq_state* s) {
    if (s->pos + 1 < s->blen) s->pos++;
    else fq_advance(s);
}
static void fq_consume_nl(fq_state* s) {
    s->nl &= s->nl - 1;
    fq_incr(s);
    s->line++;
}

static void fastq_runs(const uint8_t* d, size_t n, tor_run_cb cb, void* user) {
    fq_state s = {0};
    s.d = d;
    s.n = n;
    if (n == 0) return;
    fq_load(&s, 0);
    bbuf run = {0};
    for (;;) {
        switch (s.line & 3) {
        case 0:
            fq_incr(&s);
            if (s.finished) goto done;
            while (s.nl == 0)
                if (fq_advance(&s)) goto done;
            s.pos = (size_t)__builtin_ctzll(s.nl);
            fq_consume_nl(&s);
            break;
        case 1: {
            uint64_t mask = (s.dna | s.nl) & (~0ull << s.pos);
            while (mask == 0) {
                if (fq_advance(&s)) goto done;
                mask = s.dna | s.nl;
            }
            s.pos = (size_t)__builtin_ctzll(mask);
            if ((1ull << s.pos) & s.nl) { fq_consume_nl(&s); continue; }
            run.n = 0;
            mask = ~s.dna & (~0ull << s.pos);
            size_t first = s.pos;
            while (mask == 0) {
                bb_put(&run, d + s.blk * 64 + s.pos, s.blen - s.pos);
                if (fq_advance(&s)) goto done; /* run reaching EOF is dropped */
                first = 0;
                mask = ~s.dna;
            }
            s.pos = (size_t)__builtin_ctzll(mask);
            bb_put(&run, d + s.blk * 64 + first, s.pos - first);
            if ((1ull << s.pos) & s.nl) fq_consume_nl(&s);
            cb(run.p, run.n, user);
            break;
        }
        case 2:
            while (s.nl == 0)
                if (fq_advance(&s)) goto done;
            s.pos = (size_t)__builtin_ctzll(s.nl);
            fq_consume_nl(&s);
            break;
        case 3:
            while (s.nl == 0)
                if (fq_advance(&s)) break;
            s.pos = s.nl ? (size_t)__builtin_ctzll(s.nl) : 64;
            fq_consume_nl(&s);
            break;
        }
    }
done:
    bb_free(&run);
}

int tor_parse_fastx(const uint8_t* data, size_t len, tor_run_cb cb, void* user) {
    if (len == 0) return -1;
    if (data[0] == '@') fastq_runs(data, len, cb, user);
    else fasta_runs(data, len, cb, user);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* ntHash (include/nt_hash.hpp). nt code of an ASCII base: (c >> 1) & 3,    */
/* i.e. A0 C1 T2 G3. Seeds are the published ntHash seeds.                  */

static const uint64_t NT_FWD[4] = {
    0x3c8bfbb395c60474ULL, 0x3193c18562a02b4cULL,
    0x295549f54be24456ULL, 0x20323ed082572324ULL};
static const uint64_t NT_REV[4] = { /* REV[b] = FWD[b ^ 2] */
    0x295549f54be24456ULL, 0x20323ed082572324ULL,
    0x3c8bfbb395c60474ULL, 0x3193c18562a02b4cULL};

static inline uint64_t rol64(uint64_t x, int s) {
    s &= 63;
    return s ? (x << s) | (x >> (64 - s)) : x;
}
static inline uint64_t ror64(uint64_t x, int s) {
    s &= 63;
    return s ? (x >> s) | (x << (64 - s)) : x;
}
static inline unsigned nt_code(uint8_t c) { return (c >> 1) & 3u; }

uint64_t tor_nthash_canonical(const uint8_t* s, int m) {
    uint64_t f = 0, r = 0;
    for (int i = 0; i < m; ++i) {
        const unsigned b = nt_code(s[i]);
        f ^= rol64(NT_FWD[b], m - 1 - i);
        r ^= rol64(NT_REV[b], i);
    }
    return f ^ r;
}

/* Rolling state: fwd/rev of the current m-mer and its 2-bit nt codes. */
typedef struct {
    int m;
    uint64_t fwd, rev;
    uint64_t ctf[16], ctr[16]; /* roll terms indexed by (out << 2) | in */
} roller;

static void roller_setup(roller* h, int m) {
    h->m = m;
    for (int o = 0; o < 4; ++o)
        for (int i = 0; i < 4; ++i) {
            h->ctf[o * 4 + i] = rol64(NT_FWD[o], m) ^ NT_FWD[i];
            h->ctr[o * 4 + i] = ror64(NT_REV[o], 1) ^ rol64(NT_REV[i], m - 1);
        }
}
static inline void roller_roll(roller* h, unsigned out, unsigned in) {
    const unsigned idx = (out << 2) | in;
    h->fwd = rol64(h->fwd, 1) ^ h->ctf[idx];
    h->rev = ror64(h->rev, 1) ^ h->ctr[idx];
}

/* ------------------------------------------------------------------------ */
/* Two-stack sliding minimum (include/minimizer_window.hpp). H holds w+1    */
/* hashes written at decreasing indices; M_pre[i] = min(H[0..i]) computed   */
/* with strict '<' at every wrap; M_suf = running min since the wrap.       */

typedef struct {
    int k, m, w;
    roller h;
    uint64_t H[257], Mpre[257];
    uint16_t Mpre_idx[257];
    uint64_t Msuf;
    size_t Msuf_idx;
    uint64_t h0pos;
    size_t pivot;
    uint64_t lmer_out_shift;
    const uint8_t* seq; /* the run, for the outgoing base */
    size_t next;        /* index of the next base to enter */
} minwin;

static void mw_wrap(minwin* W) {
    W->Mpre[0] = W->H[0];
    W->Mpre_idx[0] = 0;
    for (int i = 1; i <= W->w; ++i) {
        const int lt = W->H[i] < W->Mpre[i - 1];
        W->Mpre[i] = lt ? W->H[i] : W->Mpre[i - 1];
        W->Mpre_idx[i] = lt ? (uint16_t)i : W->Mpre_idx[i - 1];
    }
    W->Msuf = UINT64_MAX;
    W->Msuf_idx = 0;
    W->pivot = (size_t)W->w;
}

static void mw_reset(minwin* W, const uint8_t* seq) {
    const int m = W->m, k = W->k;
    W->seq = seq;
    W->h.fwd = W->h.rev = 0;
    for (int i = 0; i < m; ++i) {
        const unsigned b = nt_code(seq[i]);
        W->h.fwd ^= rol64(NT_FWD[b], m - 1 - i);
        W->h.rev ^= rol64(NT_REV[b], i);
    }
    W->pivot = (size_t)W->w;
    W->H[W->pivot] = W->h.fwd ^ W->h.rev;
    for (int i = m; i < k; ++i) {
        roller_roll(&W->h, nt_code(seq[i - m]), nt_code(seq[i]));
        --W->pivot;
        W->H[W->pivot] = W->h.fwd ^ W->h.rev;
    }
    W->h0pos = (uint64_t)W->w;
    mw_wrap(W);
    W->next = (size_t)k;
}

static void mw_advance(minwin* W) {
    const size_t i = W->next++;
    roller_roll(&W->h, nt_code(W->seq[i - (size_t)W->m]), nt_code(W->seq[i]));
    const uint64_t hv = W->h.fwd ^ W->h.rev;
    W->H[W->pivot] = hv;
    if (hv < W->Msuf) { W->Msuf = hv; W->Msuf_idx = W->pivot; }
    if (W->pivot > 0) --W->pivot;
    else { W->h0pos += (uint64_t)W->w + 1; mw_wrap(W); }
}

static inline uint64_t mw_hash(const minwin* W) {
    const uint64_t a = W->Mpre[W->pivot];
    return a < W->Msuf ? a : W->Msuf;
}
static inline uint64_t mw_min_pos(const minwin* W) {
    if (W->Mpre[W->pivot] < W->Msuf) return W->h0pos - W->Mpre_idx[W->pivot];
    return W->h0pos + (uint64_t)W->w + 1 - W->Msuf_idx;
}

/* ------------------------------------------------------------------------ */
/* Superkmer extraction (src/partition_hash.hpp:48-101) and the record      */
/* layout (src/superkmer_io.hpp:3-19, :154-172).                            */

static inline unsigned kache_code(uint8_t c) { return ((c >> 2) ^ (c >> 1)) & 3u; }

static size_t hdr_bytes(int k, int m) { return (2 * k - m <= 255) ? 1 : 2; }

static size_t pack_record(uint8_t* out, const uint8_t* bases, size_t len,
                          size_t min_pos, size_t hb) {
    if (hb == 1) { out[0] = (uint8_t)len; out[1] = (uint8_t)min_pos; }
    else {
        const uint16_t l = (uint16_t)len, p = (uint16_t)min_pos;
        memcpy(out, &l, 2);
        memcpy(out + 2, &p, 2);
    }
    uint8_t* pk = out + 2 * hb;
    const size_t nb = (len + 3) / 4;
    memset(pk, 0, nb);
    for (size_t i = 0; i < len; ++i)
        pk[i >> 2] |= (uint8_t)(kache_code(bases[i]) << (6 - 2 * (i & 3)));
    return 2 * hb + nb;
}

void tor_superkmers_of_run(const uint8_t* run, size_t len, int k, int m,
                           uint64_t n_parts, tor_record_cb cb, void* user) {
    if (len < (size_t)k) return;
    const size_t hb = hdr_bytes(k, m);
    const size_t hdr_max = hb == 1 ? 255 : 65535;
    const uint64_t mask = n_parts - 1;
    minwin* W = (minwin*)malloc(sizeof(minwin));
    W->k = k; W->m = m; W->w = k - m;
    roller_setup(&W->h, m);
    mw_reset(W, run);
    uint8_t rec[4 + 16384 + 4];
    uint64_t prev_hash = mw_hash(W);
    uint64_t prev_min_pos = mw_min_pos(W);
    size_t sk_start = 0;
    for (size_t pos = (size_t)k; pos < len; ++pos) {
        mw_advance(W);
        const uint64_t nh = mw_hash(W);
        if (nh != prev_hash || pos - sk_start >= hdr_max) {
            const size_t sk_len = pos - sk_start;
            const size_t nbytes = pack_record(rec, run + sk_start, sk_len,
                                              (size_t)(prev_min_pos - sk_start), hb);
            cb(prev_hash & mask, rec, nbytes, prev_hash, user);
            prev_hash = nh;
            prev_min_pos = mw_min_pos(W);
            sk_start = pos - (size_t)(k - 1);
        }
    }
    const size_t sk_len = len - sk_start;
    const size_t nbytes = pack_record(rec, run + sk_start, sk_len,
                                      (size_t)(prev_min_pos - sk_start), hb);
    cb(prev_hash & mask, rec, nbytes, prev_hash, user);
    free(W);
}

/* ------------------------------------------------------------------------ */
/* K-mers: ceil(k/32) words, word 0 holds the last 32 bases, last base in   */
/* the low bits (Kmer.hpp:38-48); kache codes A0 C1 G2 T3. Canonical form = */
/* min(fwd, revcomp) comparing words high to low (Kmer.hpp:446-456).        */

typedef struct { uint64_t w[TOR_MAX_WORDS]; } kmer_t;

static inline int kcmp(const kmer_t* a, const kmer_t* b, int nw) {
    for (int i = nw - 1; i >= 0; --i)
        if (a->w[i] != b->w[i]) return a->w[i] < b->w[i] ? -1 : 1;
    return 0;
}

typedef struct {
    int k, nw;
    uint64_t top_mask; /* valid bits of word nw-1 */
    int top_shift;     /* bit offset of base k-1 inside word nw-1 */
} kgeom;

static kgeom kgeom_of(int k) {
    kgeom g;
    g.k = k;
    g.nw = (k + 31) / 32;
    const int top_bases = k - 32 * (g.nw - 1);
    g.top_mask = top_bases == 32 ? ~0ull : ((1ull << (2 * top_bases)) - 1);
    g.top_shift = 2 * (top_bases - 1);
    return g;
}

static inline void k_push_fwd(kmer_t* f, const kgeom* g, unsigned b) {
    for (int i = g->nw - 1; i > 0; --i) f->w[i] = (f->w[i] << 2) | (f->w[i - 1] >> 62);
    f->w[0] = (f->w[0] << 2) | b;
    f->w[g->nw - 1] &= g->top_mask;
}
static inline void k_push_rc(kmer_t* r, const kgeom* g, unsigned b) {
    for (int i = 0; i < g->nw - 1; ++i) r->w[i] = (r->w[i] >> 2) | (r->w[i + 1] << 62);
    r->w[g->nw - 1] >>= 2;
    r->w[g->nw - 1] |= (uint64_t)(3u - b) << g->top_shift;
}

/* ------------------------------------------------------------------------ */
/* Counting table: open addressing, linear probing.                         */

typedef struct {
    int nw;
    uint64_t cap, size;
    uint64_t* keys;  /* cap * nw */
    uint32_t* cnt;   /* cap; 0 = empty */
} ktable;

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}
static inline uint64_t khash(const kmer_t* a, int nw) {
    uint64_t h = 0x9e3779b97f4a7c15ULL;
    for (int i = 0; i < nw; ++i) h = mix64(h ^ a->w[i]);
    return h;
}

static void kt_init(ktable* t, int nw, uint64_t cap) {
    t->nw = nw;
    t->cap = cap;
    t->size = 0;
    t->keys = (uint64_t*)malloc(cap * nw * sizeof(uint64_t));
    t->cnt = (uint32_t*)calloc(cap, sizeof(uint32_t));
}
static void kt_free(ktable* t) { free(t->keys); free(t->cnt); }

static void kt_insert_n(ktable* t, const kmer_t* key, uint32_t add);

static void kt_grow(ktable* t) {
    ktable n;
    kt_init(&n, t->nw, t->cap * 2);
    kmer_t k;
    for (uint64_t i = 0; i < t->cap; ++i)
        if (t->cnt[i]) {
            memcpy(k.w, t->keys + i * t->nw, t->nw * sizeof(uint64_t));
            kt_insert_n(&n, &k, t->cnt[i]);
        }
    kt_free(t);
    *t = n;
}

static void kt_insert_n(ktable* t, const kmer_t* key, uint32_t add) {
    if ((t->size + 1) * 2 > t->cap) kt_grow(t);
    const int nw = t->nw;
    uint64_t i = khash(key, nw) & (t->cap - 1);
    for (;;) {
        if (t->cnt[i] == 0) {
            memcpy(t->keys + i * nw, key->w, nw * sizeof(uint64_t));
            t->cnt[i] = add;
            t->size++;
            return;
        }
        if (memcmp(t->keys + i * nw, key->w, nw * sizeof(uint64_t)) == 0) {
            t->cnt[i] += add; /* u32, wraps like the reference's v + 1 */
            return;
        }
        i = (i + 1) & (t->cap - 1);
    }
}

/* Count every k-mer of one record (count.hpp:71-175): unpack MSB-first kache
 * codes, roll the k-mer and its reverse complement, insert the canonical. */
static void count_record(ktable* t, const kgeom* g, const uint8_t* rec, size_t hb,
                         size_t* consumed) {
    size_t len;
    if (hb == 1) len = rec[0];
    else { uint16_t l; memcpy(&l, rec, 2); len = l; }
    const uint8_t* pk = rec + 2 * hb;
    *consumed = 2 * hb + (len + 3) / 4;
    if (len < (size_t)g->k) return;
    kmer_t f, r;
    memset(&f, 0, sizeof f);
    memset(&r, 0, sizeof r);
    for (size_t i = 0; i < len; ++i) {
        const unsigned b = (pk[i >> 2] >> (6 - 2 * (i & 3))) & 3u;
        k_push_fwd(&f, g, b);
        k_push_rc(&r, g, b);
        if (i + 1 >= (size_t)g->k)
            kt_insert_n(t, kcmp(&f, &r, g->nw) <= 0 ? &f : &r, 1);
    }
}

/* ------------------------------------------------------------------------ */
/* Pipeline over a sequence stream.                                         */

struct tor_result {
    int nw;
    uint64_t n;
    uint64_t* keys;
    uint32_t* counts;
};

struct tor_parts {
    uint8_t* data;
    uint64_t* offsets;
};

typedef struct {
    uint64_t off, len;
} span;

typedef struct {
    /* phase 1 */
    const uint8_t* seq;
    const span* runs;
    size_t r0, r1;
    int k, m;
    uint64_t n_parts;
    bbuf* parts;          /* n_parts buffers */
    uint64_t n_kmers, n_sk;
} p1_job;

static void p1_rec_cb(uint64_t pid, const uint8_t* rec, size_t nb, uint64_t mh, void* user) {
    (void)mh;
    p1_job* j = (p1_job*)user;
    bb_put(&j->parts[pid], rec, nb);
    j->n_sk++;
}

/* fn(args[t]) for t < threads, on threads th[t]; a worker whose thread cannot
 * be started runs on the calling thread instead. */
static void run_workers(void* (*fn)(void*), void* args, size_t arg_size, int threads, pthread_t* th) {
    unsigned char started[256] = {0}; /* threads <= 256 (clamp_threads) */
    for (int t = 0; t < threads; ++t) {
        void* a = (char*)args + (size_t)t * arg_size;
        if (t < 256 && pthread_create(&th[t], NULL, fn, a) == 0) started[t] = 1;
        else fn(a);
    }
    for (int t = 0; t < threads && t < 256; ++t)
        if (started[t]) pthread_join(th[t], NULL);
}

static void* p1_worker(void* arg) {
    p1_job* j = (p1_job*)arg;
    for (size_t r = j->r0; r < j->r1; ++r) {
        const span s = j->runs[r];
        j->n_kmers += s.len - (uint64_t)j->k + 1;
        tor_superkmers_of_run(j->seq + s.off, s.len, j->k, j->m, j->n_parts, p1_rec_cb, j);
    }
    return NULL;
}

typedef struct {
    p1_job* jobs;
    int nthreads;
    int k, m;
    uint64_t n_parts;
    uint64_t ci, cx;
    _Atomic uint64_t next;
    int digest_only;      /* fold the pairs into a digest instead of keeping them */
    /* per thread output */
    bbuf keys, cnts;
    uint64_t n_distinct, n_out;
} p2_ctx;

typedef struct {
    p2_ctx* c;
    bbuf keys, cnts;
    uint64_t n_distinct, n_out;
    tor_digest dg;
} p2_job;

static void* p2_worker(void* arg) {
    p2_job* pj = (p2_job*)arg;
    p2_ctx* c = pj->c;
    const kgeom g = kgeom_of(c->k);
    const size_t hb = hdr_bytes(c->k, c->m);
    for (;;) {
        const uint64_t p = atomic_fetch_add(&c->next, 1);
        if (p >= c->n_parts) break;
        uint64_t bytes = 0;
        for (int t = 0; t < c->nthreads; ++t) bytes += c->jobs[t].parts[p].n;
        if (!bytes) continue;
        ktable tab;
        uint64_t cap = 1024;
        while (cap < bytes) cap <<= 1;
        kt_init(&tab, g.nw, cap);
        for (int t = 0; t < c->nthreads; ++t) {
            const bbuf* b = &c->jobs[t].parts[p];
            size_t o = 0;
            while (o + 2 * hb <= b->n) {
                size_t used;
                count_record(&tab, &g, b->p + o, hb, &used);
                o += used;
            }
        }
        pj->n_distinct += tab.size;
        for (uint64_t i = 0; i < tab.cap; ++i) {
            const uint32_t cnt = tab.cnt[i];
            if (!cnt) continue;
            if ((uint64_t)cnt < c->ci || (uint64_t)cnt > c->cx) continue;
            pj->n_out++;
            if (c->digest_only) {
                tdg_add(&pj->dg, tab.keys + i * g.nw, g.nw, cnt);
                continue;
            }
            bb_put(&pj->keys, (const uint8_t*)(tab.keys + i * g.nw), g.nw * 8);
            bb_put(&pj->cnts, (const uint8_t*)&cnt, 4);
        }
        kt_free(&tab);
    }
    return NULL;
}

/* LSD radix sort of (key words, count) records by key, high word last. */
static void sort_result(tor_result* r) {
    const uint64_t n = r->n;
    const int nw = r->nw;
    if (n < 2) return;
    uint64_t* idx = (uint64_t*)malloc(n * sizeof(uint64_t));
    uint64_t* tmp = (uint64_t*)malloc(n * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; ++i) idx[i] = i;
    for (int w = 0; w < nw; ++w) {
        for (int pass = 0; pass < 4; ++pass) {
            const int sh = pass * 16;
            uint64_t* cnt = (uint64_t*)calloc(65537, sizeof(uint64_t));
            int trivial = 0;
            for (uint64_t i = 0; i < n; ++i)
                cnt[((r->keys[idx[i] * nw + w] >> sh) & 0xFFFF) + 1]++;
            for (int b = 0; b < 65536; ++b) if (cnt[b + 1] == n) trivial = 1;
            if (!trivial) {
                for (int b = 0; b < 65536; ++b) cnt[b + 1] += cnt[b];
                for (uint64_t i = 0; i < n; ++i) {
                    const uint64_t bk = (r->keys[idx[i] * nw + w] >> sh) & 0xFFFF;
                    tmp[cnt[bk]++] = idx[i];
                }
                uint64_t* s = idx; idx = tmp; tmp = s;
            }
            free(cnt);
        }
    }
    uint64_t* nk = (uint64_t*)malloc(n * nw * sizeof(uint64_t));
    uint32_t* nc = (uint32_t*)malloc(n * sizeof(uint32_t));
    for (uint64_t i = 0; i < n; ++i) {
        memcpy(nk + i * nw, r->keys + idx[i] * nw, nw * sizeof(uint64_t));
        nc[i] = r->counts[idx[i]];
    }
    free(r->keys); free(r->counts);
    r->keys = nk; r->counts = nc;
    free(idx); free(tmp);
}

typedef struct {
    bbuf runs; /* spans */
    int k;
    uint64_t n_runs;
} run_collect;

static void collect_spans(const uint8_t* seq, size_t len, int k, bbuf* out, uint64_t* n_runs) {
    size_t i = 0;
    while (i < len) {
        while (i < len && !is_acgt(seq[i])) ++i;
        const size_t s = i;
        while (i < len && is_acgt(seq[i])) ++i;
        if (i - s >= (size_t)k) {
            span sp = {s, i - s};
            bb_put(out, (const uint8_t*)&sp, sizeof sp);
            (*n_runs)++;
        }
    }
}

static int clamp_threads(int t) { return t < 1 ? 1 : (t > 256 ? 256 : t); }

static p1_job* run_phase1(const uint8_t* seq, size_t len, int k, int m, uint64_t n_parts,
                          int threads, uint64_t* n_runs_out) {
    bbuf sp = {0};
    uint64_t n_runs = 0;
    collect_spans(seq, len, k, &sp, &n_runs);
    const span* runs = (const span*)sp.p;
    uint64_t total = 0;
    for (uint64_t r = 0; r < n_runs; ++r) total += runs[r].len;
    p1_job* jobs = (p1_job*)calloc((size_t)threads, sizeof(p1_job));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    size_t r = 0;
    uint64_t acc = 0;
    for (int t = 0; t < threads; ++t) {
        jobs[t].seq = seq; jobs[t].runs = runs; jobs[t].k = k; jobs[t].m = m;
        jobs[t].n_parts = n_parts;
        jobs[t].parts = (bbuf*)calloc(n_parts, sizeof(bbuf));
        jobs[t].r0 = r;
        const uint64_t goal = total * (uint64_t)(t + 1) / (uint64_t)threads;
        while (r < n_runs && (acc < goal || t == threads - 1)) { acc += runs[r].len; ++r; }
        jobs[t].r1 = r;
    }
    run_workers(p1_worker, jobs, sizeof(p1_job), threads, th);
    free(th);
    /* spans no longer needed after phase 1 */
    bb_free(&sp);
    *n_runs_out = n_runs;
    return jobs;
}

static void free_phase1(p1_job* jobs, int threads, uint64_t n_parts) {
    for (int t = 0; t < threads; ++t) {
        for (uint64_t p = 0; p < n_parts; ++p) bb_free(&jobs[t].parts[p]);
        free(jobs[t].parts);
    }
    free(jobs);
}

static tor_result* count_stream_impl(const uint8_t* seq, size_t len, int k, int m,
                                     uint64_t n_parts, uint64_t ci, uint64_t cx,
                                     int threads, tor_stats* st, int sort_output, tor_digest* dg);

tor_result* tor_count_stream(const uint8_t* seq, size_t len, int k, int m,
                             uint64_t n_parts, uint64_t ci, uint64_t cx,
                             int threads, tor_stats* st) {
    return count_stream_impl(seq, len, k, m, n_parts, ci, cx, threads, st, 1, NULL);
}

tor_result* tor_count_stream_unsorted(const uint8_t* seq, size_t len, int k, int m,
                                      uint64_t n_parts, uint64_t ci, uint64_t cx,
                                      int threads, tor_stats* st) {
    return count_stream_impl(seq, len, k, m, n_parts, ci, cx, threads, st, 0, NULL);
}

/* With dg non-null the pairs are folded into *dg as they are found (memory for
 * one partition's table per thread) and the result holds no pairs. */
static tor_result* count_stream_impl(const uint8_t* seq, size_t len, int k, int m,
                                     uint64_t n_parts, uint64_t ci, uint64_t cx,
                                     int threads, tor_stats* st, int sort_output, tor_digest* dg) {
    if (k < 2 || k > 256 || m < 1 || m > 32 || m >= k) return NULL;
    if (n_parts == 0 || (n_parts & (n_parts - 1))) return NULL;
    threads = clamp_threads(threads);
    uint64_t n_runs = 0;
    p1_job* jobs = run_phase1(seq, len, k, m, n_parts, threads, &n_runs);
    p2_ctx c;
    memset(&c, 0, sizeof c);
    c.jobs = jobs; c.nthreads = threads; c.k = k; c.m = m; c.n_parts = n_parts;
    c.ci = ci; c.cx = cx;
    c.digest_only = dg != NULL;
    atomic_store(&c.next, 0);
    p2_job* pj = (p2_job*)calloc((size_t)threads, sizeof(p2_job));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; ++t) pj[t].c = &c;
    run_workers(p2_worker, pj, sizeof(p2_job), threads, th);
    free(th);
    const int nw = (k + 31) / 32;
    tor_result* r = (tor_result*)calloc(1, sizeof(tor_result));
    r->nw = nw;
    uint64_t n_out = 0, n_distinct = 0;
    for (int t = 0; t < threads; ++t) { n_out += pj[t].n_out; n_distinct += pj[t].n_distinct; }
    if (dg) {
        memset(dg, 0, sizeof *dg);
        for (int t = 0; t < threads; ++t) tdg_merge(dg, &pj[t].dg);
    }
    r->n = dg ? 0 : n_out;
    r->keys = (uint64_t*)malloc((r->n ? r->n : 1) * nw * sizeof(uint64_t));
    r->counts = (uint32_t*)malloc((r->n ? r->n : 1) * sizeof(uint32_t));
    uint64_t o = 0;
    for (int t = 0; t < threads; ++t) {
        if (!dg) {
            memcpy(r->keys + o * nw, pj[t].keys.p, pj[t].n_out * nw * 8);
            memcpy(r->counts + o, pj[t].cnts.p, pj[t].n_out * 4);
            o += pj[t].n_out;
        }
        bb_free(&pj[t].keys); bb_free(&pj[t].cnts);
    }
    free(pj);
    if (st) {
        memset(st, 0, sizeof *st);
        st->n_runs = n_runs;
        for (int t = 0; t < threads; ++t) {
            st->n_kmers += jobs[t].n_kmers;
            st->n_superkmers += jobs[t].n_sk;
            for (uint64_t p = 0; p < n_parts; ++p) st->record_bytes += jobs[t].parts[p].n;
        }
        st->n_distinct = n_distinct;
        st->n_out = n_out;
    }
    free_phase1(jobs, threads, n_parts);
    if (sort_output) sort_result(r);
    return r;
}

static void append_run(const uint8_t* run, size_t len, void* user) {
    bbuf* b = (bbuf*)user;
    bb_put(b, run, len);
    uint8_t sep = '\n';
    bb_put(b, &sep, 1);
}

tor_result* tor_count_fastx(const uint8_t* data, size_t len, int k, int m,
                            uint64_t n_parts, uint64_t ci, uint64_t cx,
                            int threads, tor_stats* st) {
    bbuf s = {0};
    if (tor_parse_fastx(data, len, append_run, &s) != 0) return NULL;
    tor_result* r = tor_count_stream(s.p ? s.p : (const uint8_t*)"", s.n, k, m, n_parts, ci, cx, threads, st);
    bb_free(&s);
    return r;
}

int tor_digest_stream(const uint8_t* seq, size_t len, int k, int m, uint64_t n_parts,
                      uint64_t ci, uint64_t cx, int threads, tor_stats* st, tor_digest* dg) {
    tor_result* r = count_stream_impl(seq, len, k, m, n_parts, ci, cx, threads, st, 0, dg);
    if (!r) return -1;
    tor_result_free(r);
    return 0;
}

int tor_digest_fastx(const uint8_t* data, size_t len, int k, int m, uint64_t n_parts,
                     uint64_t ci, uint64_t cx, int threads, tor_stats* st, tor_digest* dg) {
    bbuf s = {0};
    if (tor_parse_fastx(data, len, append_run, &s) != 0) return -1;
    const int rc = tor_digest_stream(s.p ? s.p : (const uint8_t*)"", s.n, k, m, n_parts, ci, cx,
                                     threads, st, dg);
    bb_free(&s);
    return rc;
}

void tor_digest_pairs(const uint64_t* keys, int stride, int nw, const uint32_t* counts, uint64_t n,
                      tor_digest* dg) {
    memset(dg, 0, sizeof *dg);
    for (uint64_t i = 0; i < n; ++i) tdg_add(dg, keys + i * (uint64_t)stride, nw, counts[i]);
}

void tor_result_digest(const tor_result* r, tor_digest* dg) {
    memset(dg, 0, sizeof *dg);
    for (uint64_t i = 0; i < r->n; ++i) tdg_add(dg, r->keys + i * r->nw, r->nw, r->counts[i]);
}

tor_parts* tor_partition_stream(const uint8_t* seq, size_t len, int k, int m,
                                uint64_t n_parts, int threads) {
    if (k < 2 || k > 256 || m < 1 || m > 32 || m >= k) return NULL;
    if (n_parts == 0 || (n_parts & (n_parts - 1))) return NULL;
    threads = clamp_threads(threads);
    uint64_t n_runs = 0;
    p1_job* jobs = run_phase1(seq, len, k, m, n_parts, threads, &n_runs);
    tor_parts* P = (tor_parts*)calloc(1, sizeof(tor_parts));
    P->offsets = (uint64_t*)calloc(n_parts + 1, sizeof(uint64_t));
    uint64_t total = 0;
    for (uint64_t p = 0; p < n_parts; ++p) {
        P->offsets[p] = total;
        for (int t = 0; t < threads; ++t) total += jobs[t].parts[p].n;
    }
    P->offsets[n_parts] = total;
    P->data = (uint8_t*)malloc(total ? total : 1);
    uint64_t o = 0;
    for (uint64_t p = 0; p < n_parts; ++p)
        for (int t = 0; t < threads; ++t) {
            memcpy(P->data + o, jobs[t].parts[p].p, jobs[t].parts[p].n);
            o += jobs[t].parts[p].n;
        }
    free_phase1(jobs, threads, n_parts);
    return P;
}

const uint8_t* tor_parts_data(const tor_parts* p) { return p->data; }
const uint64_t* tor_parts_offsets(const tor_parts* p) { return p->offsets; }
void tor_parts_free(tor_parts* p) { if (p) { free(p->data); free(p->offsets); free(p); } }

int tor_result_words(const tor_result* r) { return r->nw; }
uint64_t tor_result_size(const tor_result* r) { return r->n; }
const uint64_t* tor_result_keys(const tor_result* r) { return r->keys; }
const uint32_t* tor_result_counts(const tor_result* r) { return r->counts; }
void tor_result_free(tor_result* r) { if (r) { free(r->keys); free(r->counts); free(r); } }

/* ------------------------------------------------------------------------ */
/* Writers                                                                  */

static void kmer_label(const uint64_t* w, int k, char* out) {
    static const char map[4] = {'A', 'C', 'G', 'T'};
    for (int i = 0; i < k; ++i) {
        const int b = k - 1 - i; /* base index counted from the end */
        out[i] = map[(w[b >> 5] >> (2 * (b & 31))) & 3];
    }
}

int tor_write_tsv(const tor_result* r, int k, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    char line[300];
    for (uint64_t i = 0; i < r->n; ++i) {
        kmer_label(r->keys + i * r->nw, k, line);
        int n = snprintf(line + k, sizeof line - (size_t)k, "\t%u\n", r->counts[i]);
        fwrite(line, 1, (size_t)k + (size_t)n, f);
    }
    return fclose(f) == 0 ? 0 : -1;
}

static void put_be(FILE* f, uint64_t v, int n) {
    for (int i = n - 1; i >= 0; --i) fputc((int)((v >> (8 * i)) & 0xFF), f);
}
static void put_var(FILE* f, const char* name, uint64_t v) {
    fwrite(name, 1, strlen(name) + 1, f);
    put_be(f, v, 8);
}

/* KFF 1.0 container as the reference fills it (kff_output.hpp:20-57):
 * encoding A0 C1 G2 T3, unique + canonical, a 'v' section {k, max=1,
 * data_size=4}, one 'r' section with one k-mer per block: the k-mer as
 * ceil(k/4) bytes MSB-first (Kmer::write_packed_2bit_msb) then its count as
 * 4 bytes big-endian; a closing 'v' section {footer_size}. */
int tor_write_kff(const tor_result* r, int k, const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return -1;
    fwrite("KFF", 1, 3, f);
    fputc(1, f); fputc(0, f);
    fputc(0x1B, f);           /* A=00 C=01 G=10 T=11 */
    fputc(1, f); fputc(1, f); /* unique, canonical */
    put_be(f, 0, 4);          /* no metadata */
    fputc('v', f); put_be(f, 3, 8);
    put_var(f, "k", (uint64_t)k);
    put_var(f, "max", 1);
    put_var(f, "data_size", 4);
    fputc('r', f); put_be(f, r->n, 8);
    const size_t kb = ((size_t)k + 3) / 4;
    uint8_t buf[64];
    for (uint64_t i = 0; i < r->n; ++i) {
        const uint64_t* w = r->keys + i * r->nw;
        memset(buf, 0, kb);
        for (int j = 0; j < k; ++j) {
            const int b = k - 1 - j;
            const unsigned c = (unsigned)((w[b >> 5] >> (2 * (b & 31))) & 3);
            buf[j >> 2] |= (uint8_t)(c << (6 - 2 * (j & 3)));
        }
        fwrite(buf, 1, kb, f);
        put_be(f, r->counts[i], 4);
    }
    /* footer: a 'v' section holding its own size, then the KFF magic again */
    const char* nm = "footer_size";
    const uint64_t fsz = 1 + 8 + strlen(nm) + 1 + 8 + 3;
    fputc('v', f); put_be(f, 1, 8);
    put_var(f, nm, fsz);
    fwrite("KFF", 1, 3, f);
    return fclose(f) == 0 ? 0 : -1;
}
