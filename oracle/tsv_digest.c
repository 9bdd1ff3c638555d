/*
 * tsv_digest.c — digest of a tuna TSV output read from standard input.
 *
 * TEST INFRASTRUCTURE: tests/golden/make_golden.py pipes the reference
 * binary's TSV output (src/count.hpp:180-216: "<k-mer>\t<count>\n",
 * upper-case ACGT) through this program, so that outputs of billions of lines
 * can be pinned without storing or sorting them. The digest is the one of
 * tuna_digest.h; the line order does not matter.
 *
 * Usage: tsv_digest < out.tsv
 * Prints one JSON object: {"k": K, "pairs": N, "count_sum": S, "h1": "<hex>",
 * "h2": "<hex>"}. Exits 1 on a malformed line or lines of different k.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tuna_digest.h"

#define MAXK 256

static int code_of(int c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

int main(void) {
    static char buf[1 << 22];
    char line[MAXK + 32];
    size_t ll = 0;
    int k = -1;
    tor_digest d;
    memset(&d, 0, sizeof d);
    size_t got;
    unsigned long long lineno = 0;
    while ((got = fread(buf, 1, sizeof buf, stdin)) > 0) {
        for (size_t i = 0; i < got; ++i) {
            const char c = buf[i];
            if (c != '\n') {
                if (ll + 1 >= sizeof line) {
                    fprintf(stderr, "tsv_digest: line %llu too long\n", lineno + 1);
                    return 1;
                }
                line[ll++] = c;
                continue;
            }
            ++lineno;
            line[ll] = 0;
            char* tab = memchr(line, '\t', ll);
            if (!tab) {
                fprintf(stderr, "tsv_digest: line %llu has no tab\n", lineno);
                return 1;
            }
            const int kl = (int)(tab - line);
            if (k < 0) k = kl;
            if (kl != k || k < 1 || k > MAXK) {
                fprintf(stderr, "tsv_digest: line %llu: k-mer of length %d (expected %d)\n", lineno, kl, k);
                return 1;
            }
            uint64_t w[MAXK / 32];
            const int nw = (k + 31) / 32;
            memset(w, 0, sizeof w);
            for (int j = 0; j < k; ++j) {
                const int v = code_of(line[j]);
                if (v < 0) {
                    fprintf(stderr, "tsv_digest: line %llu: byte %d is not ACGT\n", lineno, j);
                    return 1;
                }
                const int b = k - 1 - j; /* base index counted from the end */
                w[b >> 5] |= (uint64_t)v << (2 * (b & 31));
            }
            char* end = NULL;
            const unsigned long long cnt = strtoull(tab + 1, &end, 10);
            if (end == tab + 1 || *end != 0 || cnt > 0xFFFFFFFFull) {
                fprintf(stderr, "tsv_digest: line %llu: bad count\n", lineno);
                return 1;
            }
            tdg_add(&d, w, nw, (uint32_t)cnt);
            ll = 0;
        }
    }
    if (ll) {
        fprintf(stderr, "tsv_digest: last line has no newline\n");
        return 1;
    }
    printf("{\"k\": %d, \"pairs\": %llu, \"count_sum\": %llu, \"h1\": \"%016llx\", \"h2\": \"%016llx\"}\n",
           k, (unsigned long long)d.pairs, (unsigned long long)d.count_sum, (unsigned long long)d.h1,
           (unsigned long long)d.h2);
    return 0;
}
