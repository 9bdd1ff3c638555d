/*
 * tuna_digest.h — order-independent digest of a set of (k-mer, count) pairs.
 *
 * TEST INFRASTRUCTURE: the oracle (tuna_oracle.c) and the TSV digester
 * (tsv_digest.c) use this to compare outputs that are too large to sort and
 * diff: the reference's TSV, the oracle's pairs and the GPU library's pairs
 * (which computes the same digest with its own code, tg_job_result_digest).
 *
 * The reference's output contract is the multiset of (canonical k-mer, count)
 * lines (src/count.hpp:180-216), in no particular order. Each pair is mapped
 * to two 64-bit terms and the terms are summed mod 2^64, so the digest does
 * not depend on the order of the pairs:
 *
 *   words w[0..nw), nw = ceil(k/32), in the layout of kache_hash::Kmer<k>
 *   (include/kache-hash/Kmer.hpp:38-48): word 0 holds the last 32 bases, the
 *   last base in the two low bits, codes A0 C1 G2 T3.
 *   a = 0x243F6A8885A308D3; b = 0x13198A2E03707344
 *   for i in 0..nw-1: a = fa(a ^ w[i]); b = fb(b + w[i])
 *   a = fa(a ^ (count | 1 << 40)); b = fb(b + (count ^ 0xA4093822299F31D0))
 *   h1 += a; h2 += b; pairs += 1; count_sum += count
 *
 * fa is MurmurHash3's 64-bit finaliser and fb SplitMix64's (both public
 * domain). A mis-keyed, merged, split, dropped or duplicated pair changes
 * h1 and h2 except with probability about 2^-64 each.
 */
#ifndef TUNA_DIGEST_H
#define TUNA_DIGEST_H

#include <stdint.h>

typedef struct {
    uint64_t pairs, count_sum, h1, h2;
} tor_digest;

static inline uint64_t tdg_fa(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

static inline uint64_t tdg_fb(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

static inline void tdg_add(tor_digest* d, const uint64_t* w, int nw, uint32_t count) {
    uint64_t a = 0x243F6A8885A308D3ULL, b = 0x13198A2E03707344ULL;
    for (int i = 0; i < nw; ++i) {
        a = tdg_fa(a ^ w[i]);
        b = tdg_fb(b + w[i]);
    }
    a = tdg_fa(a ^ ((uint64_t)count | (1ULL << 40)));
    b = tdg_fb(b + ((uint64_t)count ^ 0xA4093822299F31D0ULL));
    d->h1 += a;
    d->h2 += b;
    d->pairs += 1;
    d->count_sum += count;
}

static inline void tdg_merge(tor_digest* d, const tor_digest* o) {
    d->pairs += o->pairs;
    d->count_sum += o->count_sum;
    d->h1 += o->h1;
    d->h2 += o->h2;
}

#endif
