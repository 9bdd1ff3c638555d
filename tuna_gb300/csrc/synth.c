/*
 * synth.c — seeded synthetic genomes and reads for the benchmark workloads.
 *
 * Every byte depends only on (seed, parameters): the output is split into
 * fixed 1 MiB chunks, each drawn from its own splitmix64/xoshiro256** stream
 * keyed by (seed, stream id, chunk index), so the thread count changes nothing
 * and x86 and Arm hosts produce identical files (integer draws; the few double
 * thresholds are plain IEEE products, compiled with -ffp-contract=off).
 *
 *   synth_genome      i.i.d. bases at a GC fraction, optionally with interspersed
 *                     repeat families (copies mutated at a per-copy divergence)
 *                     and microsatellites (tandem units of 1-6 bp)
 *   synth_reads_fastq reads sampled uniformly from both strands of a genome,
 *                     substitution errors and N bases, Phred-30 FASTQ
 *   synth_fasta       a genome split into contigs, 60-column FASTA
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define CHUNK (1u << 20)

/* ---- PRNG: splitmix64 seeding, xoshiro256** generation ------------------ */
typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static void rng_seed(rng_t* r, uint64_t seed, uint64_t stream, uint64_t chunk) {
    uint64_t x = seed * 0x2545F4914F6CDD1DULL ^ (stream << 40) ^ chunk;
    for (int i = 0; i < 4; ++i) r->s[i] = splitmix64(&x);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t rng_next(rng_t* r) {
    const uint64_t res = rotl(r->s[1] * 5, 7) * 9;
    const uint64_t t = r->s[1] << 17;
    r->s[2] ^= r->s[0]; r->s[3] ^= r->s[1];
    r->s[1] ^= r->s[2]; r->s[0] ^= r->s[3];
    r->s[2] ^= t;
    r->s[3] = rotl(r->s[3], 45);
    return res;
}
/* uniform in [0, n) (n < 2^32), multiply-shift */
static inline uint32_t rng_below(rng_t* r, uint32_t n) {
    return (uint32_t)(((rng_next(r) >> 32) * (uint64_t)n) >> 32);
}
static inline double rng_unit(rng_t* r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* ---- base tables -------------------------------------------------------- */
static const uint8_t BASES[4] = {'A', 'C', 'G', 'T'};
static inline uint32_t base_idx(uint8_t c) {
    return c == 'A' ? 0u : c == 'C' ? 1u : c == 'G' ? 2u : 3u;
}
/* a base different from c, uniformly among the other three (r3 in [0,3)) */
static inline uint8_t other_base(uint8_t c, uint32_t r3) { return BASES[(base_idx(c) + 1 + r3) & 3]; }
static inline uint8_t comp(uint8_t c) {
    switch (c) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; case 'T': return 'A'; }
    return c;
}

/* Draw one base at GC fraction gc; a 16-bit threshold draw per base. */
typedef struct { uint32_t t_c, t_g, t_t; } gc_thr;
static gc_thr gc_thresholds(double gc) {
    gc_thr t;
    const double at = (1.0 - gc) / 2, cg = gc / 2;
    t.t_c = (uint32_t)(at * 65536.0);              /* A below */
    t.t_g = (uint32_t)((at + cg) * 65536.0);       /* C below */
    t.t_t = (uint32_t)((at + 2 * cg) * 65536.0);   /* G below, T above */
    return t;
}
static inline uint8_t draw_base(uint32_t u16, const gc_thr* t) {
    return u16 < t->t_c ? 'A' : u16 < t->t_g ? 'C' : u16 < t->t_t ? 'G' : 'T';
}
static void fill_iid(rng_t* r, uint8_t* out, size_t n, const gc_thr* t) {
    size_t i = 0;
    while (i < n) {
        uint64_t x = rng_next(r);
        for (int j = 0; j < 4 && i < n; ++j, ++i, x >>= 16) out[i] = draw_base((uint32_t)(x & 0xFFFF), t);
    }
}

/* ---- genome with repeats ------------------------------------------------ */
typedef struct {
    uint64_t seed;
    double gc;
    /* repeat families: family lengths and counts; fractions by length */
    uint32_t n_fam_a, len_a;  /* e.g. 300 bp families */
    uint32_t n_fam_b, len_b;  /* e.g. 6 kbp families */
    double frac_a, frac_b;    /* fraction of sequence covered by copies */
    double div_lo, div_hi;    /* per-copy divergence range */
    double frac_micro;        /* microsatellite fraction */
    uint32_t micro_lo, micro_hi; /* microsatellite length range */
    uint32_t bg_mean;         /* mean background segment length */
} genome_params;

typedef struct {
    const genome_params* p;
    uint8_t* out;
    uint64_t len;
    const uint8_t* fam_a; /* n_fam_a * len_a */
    const uint8_t* fam_b;
    double pr_a, pr_b, pr_m; /* per-segment type probabilities */
    uint64_t next_chunk, n_chunks;
    pthread_mutex_t mu;
} genome_job;

static void gen_chunk(genome_job* J, uint64_t c) {
    const genome_params* p = J->p;
    rng_t r;
    rng_seed(&r, p->seed, 1, c);
    const gc_thr t = gc_thresholds(p->gc);
    uint8_t* o = J->out + c * CHUNK;
    const uint64_t n = (c + 1) * CHUNK <= J->len ? CHUNK : J->len - c * CHUNK;
    uint64_t i = 0;
    while (i < n) {
        const double u = rng_unit(&r);
        uint64_t seg;
        if (u < J->pr_a || (u < J->pr_a + J->pr_b)) {
            const int is_a = u < J->pr_a;
            const uint32_t fl = is_a ? p->len_a : p->len_b;
            const uint8_t* fam = is_a ? J->fam_a + (uint64_t)rng_below(&r, p->n_fam_a) * fl
                                      : J->fam_b + (uint64_t)rng_below(&r, p->n_fam_b) * fl;
            const double div = p->div_lo + (p->div_hi - p->div_lo) * rng_unit(&r);
            const uint32_t thr = (uint32_t)(div * 4294967296.0);
            const int rc = (int)(rng_next(&r) & 1);
            seg = fl;
            if (seg > n - i) seg = n - i;
            for (uint64_t j = 0; j < seg; ++j) {
                uint8_t b = rc ? comp(fam[fl - 1 - j]) : fam[j];
                if ((uint32_t)(rng_next(&r) >> 32) < thr) b = other_base(b, rng_below(&r, 3));
                o[i + j] = b;
            }
        } else if (u < J->pr_a + J->pr_b + J->pr_m) {
            const uint32_t unit = 1 + rng_below(&r, 6);
            uint8_t motif[6];
            for (uint32_t j = 0; j < unit; ++j) motif[j] = BASES[rng_below(&r, 4)];
            seg = p->micro_lo + rng_below(&r, p->micro_hi - p->micro_lo + 1);
            if (seg > n - i) seg = n - i;
            for (uint64_t j = 0; j < seg; ++j) o[i + j] = motif[j % unit];
        } else {
            /* background segment, uniform in [bg_mean/2, 3*bg_mean/2] */
            seg = p->bg_mean / 2 + rng_below(&r, p->bg_mean + 1);
            if (seg > n - i) seg = n - i;
            fill_iid(&r, o + i, seg, &t);
        }
        i += seg;
    }
}

static void* genome_worker(void* arg) {
    genome_job* J = (genome_job*)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const uint64_t c = J->next_chunk++;
        pthread_mutex_unlock(&J->mu);
        if (c >= J->n_chunks) break;
        gen_chunk(J, c);
    }
    return NULL;
}

/* fn pulls chunks from the job's shared counter: if a thread cannot be
 * started, the calling thread runs fn too and the started ones share the rest. */
static void run_threads(void* (*fn)(void*), void* job, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    int started[256];
    int missing = 0;
    for (int i = 0; i < threads; ++i) {
        started[i] = pthread_create(&th[i], NULL, fn, job) == 0;
        missing |= !started[i];
    }
    if (missing) fn(job);
    for (int i = 0; i < threads; ++i)
        if (started[i]) pthread_join(th[i], NULL);
}

/* Returns 0. out must hold len bytes. Repeat parameters of zero disable. */
int synth_genome(uint8_t* out, uint64_t len, uint64_t seed, double gc,
                 uint32_t n_fam_a, uint32_t len_a, double frac_a,
                 uint32_t n_fam_b, uint32_t len_b, double frac_b,
                 double div_lo, double div_hi,
                 double frac_micro, uint32_t micro_lo, uint32_t micro_hi,
                 int threads) {
    genome_params p;
    memset(&p, 0, sizeof p);
    p.seed = seed; p.gc = gc;
    p.n_fam_a = n_fam_a; p.len_a = len_a; p.frac_a = n_fam_a ? frac_a : 0;
    p.n_fam_b = n_fam_b; p.len_b = len_b; p.frac_b = n_fam_b ? frac_b : 0;
    p.div_lo = div_lo; p.div_hi = div_hi;
    p.frac_micro = frac_micro; p.micro_lo = micro_lo ? micro_lo : 20; p.micro_hi = micro_hi ? micro_hi : 200;
    p.bg_mean = 2000;
    /* family consensus sequences from their own stream */
    rng_t r;
    rng_seed(&r, seed, 2, 0);
    const gc_thr t = gc_thresholds(gc);
    uint8_t* fa = (uint8_t*)malloc((size_t)n_fam_a * len_a + 1);
    uint8_t* fb = (uint8_t*)malloc((size_t)n_fam_b * len_b + 1);
    fill_iid(&r, fa, (size_t)n_fam_a * len_a, &t);
    fill_iid(&r, fb, (size_t)n_fam_b * len_b, &t);
    /* segment-type probabilities from length fractions */
    const double mean_m = 0.5 * (p.micro_lo + p.micro_hi);
    const double frac_bg = 1.0 - p.frac_a - p.frac_b - p.frac_micro;
    const double wa = p.frac_a / (len_a ? len_a : 1), wb = p.frac_b / (len_b ? len_b : 1);
    const double wm = p.frac_micro / mean_m, wg = frac_bg / p.bg_mean;
    const double ws = wa + wb + wm + wg;
    genome_job J;
    memset(&J, 0, sizeof J);
    J.p = &p; J.out = out; J.len = len; J.fam_a = fa; J.fam_b = fb;
    J.pr_a = wa / ws; J.pr_b = wb / ws; J.pr_m = wm / ws;
    J.n_chunks = (len + CHUNK - 1) / CHUNK;
    pthread_mutex_init(&J.mu, NULL);
    run_threads(genome_worker, &J, threads);
    pthread_mutex_destroy(&J.mu);
    free(fa); free(fb);
    return 0;
}

/* ---- reads -------------------------------------------------------------- */
/* FASTQ record: "@r<12 digits>\n" seq "\n+\n" qual "\n". Read lengths fixed
 * (len_lo == len_hi) or uniform in [len_lo, len_hi]. Returns the bytes needed
 * when out is NULL (an upper bound), else the bytes written. */
typedef struct {
    const uint8_t* genome;
    uint64_t glen;
    uint64_t n_reads;
    uint32_t len_lo, len_hi;
    double err, n_rate;
    uint64_t seed;
    uint8_t* out;
    uint64_t* rec_off;  /* per-chunk output offsets (n_read_chunks + 1) */
    uint64_t read_chunk; /* reads per chunk */
    uint64_t next, n_chunks;
    int pass; /* 0: sizes, 1: write */
    pthread_mutex_t mu;
} reads_job;

#define READS_PER_CHUNK 8192u

static uint64_t read_len_of(rng_t* r, const reads_job* J) {
    return J->len_lo == J->len_hi ? J->len_lo : J->len_lo + rng_below(r, J->len_hi - J->len_lo + 1);
}

static void reads_chunk(reads_job* J, uint64_t c) {
    rng_t r, rl;
    rng_seed(&r, J->seed, 3, c);
    rng_seed(&rl, J->seed, 4, c);  /* read lengths: their own stream, the same in both passes */
    const uint64_t r0 = c * READS_PER_CHUNK;
    const uint64_t r1 = r0 + READS_PER_CHUNK < J->n_reads ? r0 + READS_PER_CHUNK : J->n_reads;
    if (J->pass == 0) {
        uint64_t bytes = 0;
        for (uint64_t i = r0; i < r1; ++i) {
            const uint64_t L = read_len_of(&rl, J);
            bytes += 15 + 2 * L + 4; /* "@r" + 12 digits + LF, seq, "\n+\n", qual, LF */
        }
        J->rec_off[c + 1] = bytes;
        return;
    }
    uint8_t* o = J->out + J->rec_off[c];
    const uint32_t te = (uint32_t)(J->err * 4294967296.0);
    const uint32_t tn = (uint32_t)(J->n_rate * 4294967296.0);
    for (uint64_t i = r0; i < r1; ++i) {
        const uint64_t L = read_len_of(&rl, J);
        const uint64_t pos = (rng_next(&r) >> 11) % (J->glen - L + 1);
        const int rc = (int)(rng_next(&r) & 1);
        *o++ = '@'; *o++ = 'r';
        uint64_t id = i;
        for (int d = 11; d >= 0; --d) { o[d] = (uint8_t)('0' + id % 10); id /= 10; }
        o += 12;
        *o++ = '\n';
        for (uint64_t j = 0; j < L; ++j) {
            uint8_t b = rc ? comp(J->genome[pos + L - 1 - j]) : J->genome[pos + j];
            const uint64_t x = rng_next(&r);
            if ((uint32_t)x < te) b = other_base(b, (uint32_t)(((x >> 32) & 0xFFFF) * 3 >> 16));
            if (tn && (uint32_t)(rng_next(&r) >> 32) < tn) b = 'N';
            o[j] = b;
        }
        o += L;
        *o++ = '\n'; *o++ = '+'; *o++ = '\n';
        memset(o, '?', L);
        o += L;
        *o++ = '\n';
    }
}

static void* reads_worker(void* arg) {
    reads_job* J = (reads_job*)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const uint64_t c = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (c >= J->n_chunks) break;
        reads_chunk(J, c);
    }
    return NULL;
}

/* Two calls: first with out == NULL returns the exact byte count; the second
 * writes the FASTQ into out. */
uint64_t synth_reads_fastq(const uint8_t* genome, uint64_t glen, uint64_t n_reads,
                           uint32_t len_lo, uint32_t len_hi, double err, double n_rate,
                           uint64_t seed, uint8_t* out, int threads) {
    if (glen < len_hi || n_reads == 0) return 0;
    reads_job J;
    memset(&J, 0, sizeof J);
    J.genome = genome; J.glen = glen; J.n_reads = n_reads;
    J.len_lo = len_lo; J.len_hi = len_hi; J.err = err; J.n_rate = n_rate;
    J.seed = seed; J.out = out;
    J.n_chunks = (n_reads + READS_PER_CHUNK - 1) / READS_PER_CHUNK;
    J.rec_off = (uint64_t*)calloc(J.n_chunks + 1, sizeof(uint64_t));
    pthread_mutex_init(&J.mu, NULL);
    J.pass = 0;
    run_threads(reads_worker, &J, threads);
    for (uint64_t c = 0; c < J.n_chunks; ++c) J.rec_off[c + 1] += J.rec_off[c];
    const uint64_t total = J.rec_off[J.n_chunks];
    if (out) {
        J.pass = 1;
        J.next = 0;
        run_threads(reads_worker, &J, threads);
    }
    pthread_mutex_destroy(&J.mu);
    free(J.rec_off);
    return total;
}

/* ---- FASTA -------------------------------------------------------------- */
/* contig c of length lens[c] takes the next lens[c] genome bases; header
 * ">contig_<c>\n", 60 bases per line. Returns bytes needed / written. */
uint64_t synth_fasta(const uint8_t* genome, const uint64_t* lens, uint32_t n_contigs,
                     uint8_t* out) {
    uint64_t o = 0, g = 0;
    for (uint32_t c = 0; c < n_contigs; ++c) {
        char hdr[32];
        int hl = 0;
        hdr[hl++] = '>';
        memcpy(hdr + hl, "contig_", 7); hl += 7;
        char num[12]; int nl = 0; uint32_t v = c;
        do { num[nl++] = (char)('0' + v % 10); v /= 10; } while (v);
        while (nl) hdr[hl++] = num[--nl];
        hdr[hl++] = '\n';
        if (out) memcpy(out + o, hdr, (size_t)hl);
        o += (uint64_t)hl;
        for (uint64_t i = 0; i < lens[c]; i += 60) {
            const uint64_t n = lens[c] - i < 60 ? lens[c] - i : 60;
            if (out) { memcpy(out + o, genome + g + i, n); out[o + n] = '\n'; }
            o += n + 1;
        }
        g += lens[c];
    }
    return o;
}
