/*
 * tuna_oracle.h — CPU restatement of the reference tuna counting path.
 *
 * TEST INFRASTRUCTURE, NOT THE PRODUCT. Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library, and only to verify
 * results (or as the timed CPU baseline). The GPU library never links or calls it.
 *
 * Every stage follows one function of the reference (paths are relative to
 * the reference project root):
 *   parse       include/helicase_cpp/lexer.hpp:46-68, parser_fasta.hpp:233-316,
 *               parser_fastq.hpp:112-285, simd.hpp:299-343, seq_source.hpp:169-204
 *   ntHash      include/nt_hash.hpp:26-40, :74-124
 *   minimizer   include/minimizer_window.hpp:24-200 (two-stack window, kept
 *               stateful so that min_pos ties come out exactly as the reference's)
 *   superkmers  src/partition_hash.hpp:48-101, partition fn :550-552
 *   records     src/superkmer_io.hpp:3-19, :47-52, :154-172
 *   counting    src/count.hpp:71-175 (+ Kmer.hpp:446-456 canonical order)
 *   output      src/count.hpp:180-216 (TSV), :224-265 + kff_output.hpp (KFF)
 */
#ifndef TUNA_ORACLE_H
#define TUNA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TOR_MAX_WORDS 8 /* k <= 256 */

/* Called once per maximal ACGT run, in input order. */
typedef void (*tor_run_cb)(const uint8_t* run, size_t len, void* user);

/* Parse a FASTA or FASTQ byte buffer (FASTQ iff data[0] == '@'). Returns 0,
 * or -1 for an empty buffer (the reference throws "Empty file"). */
int tor_parse_fastx(const uint8_t* data, size_t len, tor_run_cb cb, void* user);

/* Canonical ntHash (fwd ^ rev) of the m-mer at s (ASCII ACGT, any case). */
uint64_t tor_nthash_canonical(const uint8_t* s, int m);

/* Phase 1 on one run: emit every superkmer record of the run.
 * rec = [hdr len][hdr min_pos][packed bases], hdr is u8 when 2k-m <= 255. */
typedef void (*tor_record_cb)(uint64_t pid, const uint8_t* rec, size_t rec_bytes,
                              uint64_t min_hash, void* user);
void tor_superkmers_of_run(const uint8_t* run, size_t len, int k, int m,
                           uint64_t n_parts, tor_record_cb cb, void* user);

/* Whole pipeline over a sequence stream: any byte outside [ACGTacgt] separates
 * runs (this is the same input convention the GPU library takes).
 * Results are sorted by canonical k-mer (words compared high to low).
 * keys: n_out * words u64 (word 0 = last 32 bases, as Kmer<k>); counts: n_out. */
typedef struct {
    uint64_t n_runs;        /* runs of length >= k */
    uint64_t n_kmers;       /* k-mer instances */
    uint64_t n_superkmers;  /* records */
    uint64_t n_distinct;    /* distinct canonical k-mers before ci/cx */
    uint64_t n_out;         /* after ci/cx */
    uint64_t record_bytes;  /* total record bytes over all partitions */
} tor_stats;

typedef struct tor_result tor_result;
tor_result* tor_count_stream(const uint8_t* seq, size_t len, int k, int m,
                             uint64_t n_parts, uint64_t ci, uint64_t cx,
                             int threads, tor_stats* st);
/* Same without the final sort (the reference's own output is unsorted); the
 * CPU baseline times this one. */
tor_result* tor_count_stream_unsorted(const uint8_t* seq, size_t len, int k, int m,
                                      uint64_t n_parts, uint64_t ci, uint64_t cx,
                                      int threads, tor_stats* st);
/* Same, but parses FASTA/FASTQ bytes first (helicase semantics). */
tor_result* tor_count_fastx(const uint8_t* data, size_t len, int k, int m,
                            uint64_t n_parts, uint64_t ci, uint64_t cx,
                            int threads, tor_stats* st);
int tor_result_words(const tor_result* r);
uint64_t tor_result_size(const tor_result* r);
const uint64_t* tor_result_keys(const tor_result* r);
const uint32_t* tor_result_counts(const tor_result* r);
void tor_result_free(tor_result* r);

/* Order-independent digest of the pairs (tuna_digest.h defines it). The
 * *_digest_* pipelines keep no pairs: memory for Phase 1's records and one
 * partition table per thread. Return 0, or -1 for rejected parameters / an
 * empty FASTX buffer. */
#include "tuna_digest.h"
int tor_digest_stream(const uint8_t* seq, size_t len, int k, int m, uint64_t n_parts,
                      uint64_t ci, uint64_t cx, int threads, tor_stats* st, tor_digest* dg);
int tor_digest_fastx(const uint8_t* data, size_t len, int k, int m, uint64_t n_parts,
                     uint64_t ci, uint64_t cx, int threads, tor_stats* st, tor_digest* dg);
void tor_result_digest(const tor_result* r, tor_digest* dg);
/* Digest of n pairs held in arrays: pair i's words are keys[i * stride ..
 * i * stride + nw) (nw = ceil(k/32) <= stride). */
void tor_digest_pairs(const uint64_t* keys, int stride, int nw, const uint32_t* counts, uint64_t n,
                      tor_digest* dg);

/* Phase 1 only: partition contents in the reference's record layout.
 * Returns a buffer of all records grouped by partition; offsets[n_parts + 1]. */
typedef struct tor_parts tor_parts;
tor_parts* tor_partition_stream(const uint8_t* seq, size_t len, int k, int m,
                                uint64_t n_parts, int threads);
const uint8_t* tor_parts_data(const tor_parts* p);
const uint64_t* tor_parts_offsets(const tor_parts* p);
void tor_parts_free(tor_parts* p);

/* Writers over a result. Return 0 or -1 on I/O error. */
int tor_write_tsv(const tor_result* r, int k, const char* path);
int tor_write_kff(const tor_result* r, int k, const char* path);

#ifdef __cplusplus
}
#endif
#endif
