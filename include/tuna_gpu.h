/*
 * tuna_gpu.h — C ABI of the GB300 k-mer counting library (libtuna_gpu.so).
 *
 * Drop-in boundary for tuna's two-phase counting path. The reference runs the
 * path inside C++ templates; each entry point below replaces one piece of it
 * (paths relative to the reference project root):
 *
 *   tg_ctx_create / tg_ctx_destroy   the worker-thread pools and per-thread
 *                                    tables of src/count.hpp:720-970 and
 *                                    src/partition_hash.hpp:259-338
 *   tg_job_begin                     Config (src/Config.hpp:10-26) + the
 *                                    partition count of include/tuna/tuna.hpp:116-119
 *   tg_job_feed_fastx / _file /      SeqSource::process (src/seq_source.hpp:190-205) and
 *     _fastx_device                    the helicase parsers (lexed on the device)
 *   tg_read_input                    the file reading of SeqSource and GzInput
 *                                    (src/seq_source.hpp:48-141, :196-204)
 *   tg_fastx_to_stream               the helicase parsers alone (include/helicase_cpp/)
 *   tg_job_feed_seq / _seq_device    the ACTG chunks handed to
 *                                    extract_superkmers_from_actg (src/partition_hash.hpp:48)
 *   tg_job_run                       run<k,m> / run_callback<k,m> phases 1+2
 *                                    (src/pipeline.hpp:64-330)
 *   tg_job_drain                     write_counts / write_counts_kff /
 *                                    write_counts_callback (src/count.hpp:180-298)
 *   tg_job_result_copy               count_to_raw (include/tuna/tuna.hpp:181-195)
 *   tg_job_result_digest             no counterpart: a checksum of the output lines of
 *                                    write_counts (src/count.hpp:180-216), any order
 *   tg_job_export_partitions         the hash_<p>.superkmers files of the disk
 *                                    pipeline (src/superkmer_io.hpp:3-19, -tp -kt)
 *   tg_job_stats                     the phase1:/phase2:/superkmers:/unique_kmers:
 *                                    stderr lines (src/pipeline.hpp:174-178)
 *   tg_count_seq / tg_count_fastx    one call: feed, run_callback, count_to_raw
 *   tg_count_batch / _batch_fastx,   no counterpart (the reference counts one input
 *     tg_job_next_sample             set per run): several samples in one pass
 *   hbm_budget_bytes (phase 2 in     the disk mode of src/pipeline.hpp:186-263
 *     passes)
 *   tg_job_set_spill                 the disk pipeline: per-partition superkmer files
 *                                    (src/pipeline.hpp:186-263, src/superkmer_io.hpp:154-266)
 *   tg_job_set_shard                 the partitions one worker takes in phase 2
 *                                    (src/count.hpp:322-336), as a static share per
 *                                    device: the partition -> device map
 *
 * Conventions: every function returns a tg_status (0 = ok); no exception
 * crosses the ABI; tg_last_error() gives the message of the last failure on a
 * context. A context is owned by one host thread at a time; jobs of one
 * context run in submission order on its stream.
 *
 * Input convention of the *_seq entry points: a byte stream in which every
 * byte outside [ACGTacgt] separates runs (the ACGT-only chunks of the
 * reference's parser). Runs never continue across two feed calls.
 *
 * Output: canonical k-mers as ceil((k+1)/32) little-endian u64 words with
 * the layout of tuna::Kmer<k> (word 0 holds the last 32 bases, last base in
 * the two low bits, kache codes A0 C1 G2 T3), and u32 counts. For k <= 31
 * that is one word per k-mer, for 32 <= k <= 63 two.
 */
#ifndef TUNA_GPU_H
#define TUNA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TG_OK = 0,
    TG_ERR_ARG = 1,        /* bad parameter (k, m, n, sizes, null pointers) */
    TG_ERR_CUDA = 2,       /* a CUDA call failed; see tg_last_error */
    TG_ERR_OOM = 3,        /* device, pinned or host memory (or host threads) exhausted;
                              a host-side C++ failure is reported as this, "host: ..." */
    TG_ERR_STATE = 4,      /* call out of order (e.g. feed after run) */
    TG_ERR_IO = 5,         /* file could not be opened / read / written */
    TG_ERR_PARSE = 6,      /* empty input file ("Empty file") */
    TG_ERR_TABLE = 7,      /* a counting table could not hold a partition */
    TG_ERR_DEVICE = 8,     /* a device-side wait gave up (bounded spin) */
    TG_ERR_UNSUPPORTED = 9 /* parameters valid for tuna but not on this GPU path */
} tg_status;

typedef struct tg_ctx tg_ctx;
typedef struct tg_job tg_job;

typedef struct {
    int device;                 /* CUDA device ordinal */
    uint64_t hbm_budget_bytes;  /* device memory phase 2 may hold at once (keys, pairs, groups);
                                   0 = free HBM minus a reserve. A job whose keys and pairs do
                                   not fit is counted in passes over ranges of bins, each pass's
                                   pairs copied to host memory (results then stay on the host) */
    uint32_t host_threads;      /* host parser / formatter threads; 0 = all cores */
    uint32_t flags;             /* TG_CTX_* bits */
} tg_ctx_opts;

/* tg_ctx_opts.flags: the first job of each key width (k <= 31, k >= 32) with at
 * least 2^26 k-mers times its counting pass with several group sizes (the load
 * of the shared-memory table when a group's keys are all distinct) on its own
 * keys and keeps the fastest for itself and every later job of the context
 * (tg_stats.group_load_pct). Without it the group size is half the table. */
#define TG_CTX_AUTOTUNE 1u

typedef struct {
    uint16_t k;          /* 2..63 on this path */
    uint16_t m;          /* 1..min(k-1, 32) */
    uint32_t n_parts;    /* tuna -n: power of two, used for exported partition
                            files and reported; 0 = 16 */
    uint64_t ci;         /* keep k-mers with ci <= count <= cx */
    uint64_t cx;
    uint32_t gpu_parts;  /* internal bucket count (power of two); 0 = auto */
    uint32_t flags;      /* reserved, 0 */
} tg_job_opts;

typedef struct {
    uint64_t input_bytes;     /* bytes fed (sequence stream bytes) */
    uint64_t bases;           /* ACGT bases fed */
    uint64_t runs;            /* ACGT runs of length >= k */
    uint64_t kmers;           /* k-mer instances */
    uint64_t superkmers;      /* superkmer records (reference's superkmers:) */
    uint64_t distinct;        /* distinct canonical k-mers before ci/cx */
    uint64_t out;             /* k-mers after ci/cx (reference's unique_kmers:) */
    uint32_t gpu_parts;       /* internal bucket count used */
    uint32_t heavy_groups;    /* phase-2 groups larger than one table's target */
    uint64_t fallback_groups; /* key ranges counted in a global-memory table */
    double h2d_ms;            /* host->device copy time of the input */
    double pack_ms;           /* device time: 2-bit packing */
    double phase1_ms;         /* device time: minimizers, superkmers, bin histogram */
    double phase2_ms;         /* device time: counting, filter, compaction */
    double d2h_ms;            /* device->host time of results (copy / drain) */
    double phase1_cut_ms;     /* part of phase1_ms: the superkmer cut kernel */
    double phase1_scatter_ms; /* part of phase1_ms: the bucket scatter kernel */
    uint64_t record_bytes;    /* bytes of bucket records written */
    uint64_t gpu_launches;    /* kernels launched by the last tg_job_run */
    double phase2_count_ms;   /* part of phase2_ms: the shared-memory counting kernel(s) */
    double phase2_keys_ms;    /* part of phase2_ms: bin histogram, group plan, key array */
    uint64_t groups;          /* phase-2 groups (runs of minimizer bins counted in one table) */
    double lex_ms;            /* device time: FASTA/FASTQ lexing of the feeds */
    uint64_t fastx_bytes;     /* FASTA/FASTQ bytes fed (before lexing) */
    uint64_t host_parsed_bytes; /* of those, bytes parsed on the host (see tg_job_feed_fastx) */
    uint64_t phase2_passes;   /* phase-2 passes over ranges of bins (more than 1 when the keys and
                                 pairs of a job exceed the context's memory budget, hbm_budget_bytes) */
    uint32_t group_load_pct;  /* keys per counting group, % of the shared-memory table's slots */
    uint32_t autotune_trials; /* counting passes this job timed for TG_CTX_AUTOTUNE */
} tg_stats;

/* Output formats of tg_job_drain. */
typedef enum {
    TG_FMT_TSV = 0,   /* "<kmer>\t<count>\n", as write_counts (count.hpp:180-216) */
    TG_FMT_KFF = 1,   /* KFF raw section body: ceil(k/4) B MSB-first + u32 BE */
    TG_FMT_RAW = 2    /* words u64 x ceil((k+1)/32) then u32 count, packed */
} tg_format;

/* Sink of tg_job_drain: called with consecutive output chunks from the
 * calling thread; return 0 to continue, non-zero to stop with TG_ERR_IO. */
typedef int (*tg_sink_fn)(const void* data, size_t bytes, uint64_t n_kmers, void* user);

/* ---- context ---------------------------------------------------------- */
tg_status tg_ctx_create(const tg_ctx_opts* opts, tg_ctx** out);
tg_status tg_ctx_destroy(tg_ctx* ctx);
const char* tg_last_error(const tg_ctx* ctx);
/* The cudaStream_t (as void*) on which the context launches all its work, so a
 * caller can order its own work and time with CUDA events on the same stream. */
void* tg_ctx_stream(const tg_ctx* ctx);
/* Library version string and whether a CUDA device is usable. */
const char* tg_version(void);
int tg_device_count(void);

/* ---- jobs ------------------------------------------------------------- */
tg_status tg_job_begin(tg_ctx* ctx, const tg_job_opts* opts, tg_job** out);
/* Host bytes of a sequence stream (non-ACGT separates runs). */
tg_status tg_job_feed_seq(tg_job* job, const uint8_t* seq, size_t len);
/* Same, already in device memory on the context's device; the buffer must stay
 * valid and unchanged until tg_job_run returns. No copy is made. */
tg_status tg_job_feed_seq_device(tg_job* job, const uint8_t* dseq, size_t len);
/* FASTA/FASTQ bytes (FASTQ iff the first byte is '@'): copied to the device
 * and lexed there with the rules of the reference's parser
 * (include/helicase_cpp/parser_fasta.hpp:233-316, parser_fastq.hpp:112-285).
 * One case of malformed FASTQ, where the reference's 64-byte block walk departs
 * from line counting (an empty header line ending at file offset 63 mod 64),
 * is detected on the device and parsed on the host instead
 * (tg_stats.host_parsed_bytes). An empty buffer fails with TG_ERR_PARSE. */
tg_status tg_job_feed_fastx(tg_job* job, const uint8_t* data, size_t len);
/* The same for bytes already in device memory on the context's device (read
 * during the call only). */
tg_status tg_job_feed_fastx_device(tg_job* job, const uint8_t* ddata, size_t len);
/* A FASTA/FASTQ file, plain or gzip (by the ".gz" suffix): read (and
 * inflated) on the host, lexed on the device. */
tg_status tg_job_feed_file(tg_job* job, const char* path);
/* Phase 1 + Phase 2 on the device. Blocks until the counts are ready. */
tg_status tg_job_run(tg_job* job);
tg_status tg_job_stats(const tg_job* job, tg_stats* out);
/* Number of k-mers after the ci/cx filter. */
uint64_t tg_job_result_size(const tg_job* job);
/* Words per k-mer in RAW output (1 for k <= 31, 2 for k <= 63). */
int tg_job_key_words(const tg_job* job);
/* Copy results [first, first + n) to host memory (any order of k-mers, the
 * same order every call). keys: n * key_words u64; counts: n u32. */
tg_status tg_job_result_copy(tg_job* job, uint64_t* keys, uint32_t* counts,
                             uint64_t first, uint64_t n);
/* Order-independent digest of results [first, first + n): the check of an
 * output against another (the reference's TSV, a CPU count) when the outputs
 * are too large to sort and compare. The reference's output contract is the
 * multiset of (canonical k-mer, count) lines in any order (write_counts,
 * src/count.hpp:180-216); each pair maps to two 64-bit terms and the terms are
 * summed mod 2^64:
 *   words w[0..nw), nw = ceil(k/32), in the tuna::Kmer<k> layout
 *   a = 0x243F6A8885A308D3; b = 0x13198A2E03707344
 *   for i in 0..nw-1: a = fa(a ^ w[i]); b = fb(b + w[i])
 *   h1 += fa(a ^ (count | 1 << 40)); h2 += fb(b + (count ^ 0xA4093822299F31D0))
 * with fa MurmurHash3's 64-bit finaliser and fb SplitMix64's. Computed on the
 * device (or on host threads for a job whose pairs are in host memory). */
typedef struct {
    uint64_t pairs;      /* n */
    uint64_t count_sum;  /* sum of the counts */
    uint64_t h1, h2;     /* the two digests */
} tg_digest;
tg_status tg_job_result_digest(tg_job* job, uint64_t first, uint64_t n, tg_digest* out);
/* Format results on the device and hand them to sink in chunks. */
tg_status tg_job_drain(tg_job* job, tg_format fmt, tg_sink_fn sink, void* user);
/* Write results to a file: TSV, or a complete KFF file when fmt == TG_FMT_KFF. */
tg_status tg_job_write(tg_job* job, tg_format fmt, const char* path);
/* Phase 1 partitions in the reference's superkmer file layout for tuna -n
 * (job opts n_parts): sink(p, bytes, len) once per partition in order. */
typedef int (*tg_part_sink_fn)(uint32_t part, const uint8_t* data, size_t len, void* user);
tg_status tg_job_export_partitions(tg_job* job, tg_part_sink_fn sink, void* user);
tg_status tg_job_end(tg_job* job);

/* ---- several samples in one job ------------------------------------------
 * No counterpart in the reference, which counts one input set per run. A job
 * may hold up to TG_MAX_SAMPLES independent samples: feed the first, call
 * tg_job_next_sample(), feed the second, and so on. Each sample is counted on
 * its own (a k-mer present in two samples gives two pairs, each with its own
 * count), all of them in one pass of the device pipeline; the result of a
 * sample is the same as when it runs alone. The results of such a job are
 * sample-major: sample i's pairs are [offsets[i], offsets[i+1]) of
 * tg_job_result_copy, with offsets from tg_job_sample_offsets (n + 1 entries).
 * Partition export needs a job of one sample. */
#define TG_MAX_SAMPLES 65536u
tg_status tg_job_next_sample(tg_job* job);
uint32_t tg_job_sample_count(const tg_job* job);
tg_status tg_job_sample_offsets(tg_job* job, uint64_t* offsets);

/* ---- spill: jobs larger than device memory --------------------------------
 * The disk pipeline of the reference (src/pipeline.hpp:186-263: phase 1 appends
 * every superkmer to its partition's file, SuperkmerWriter::append_kache,
 * src/superkmer_io.hpp:154-172; phase 2 replays one partition file at a time,
 * SuperkmerReader, :196-266). After tg_job_set_spill, the job's input is
 * handled in chunks of at most chunk_bytes stream bytes (0 = a sixteenth of the
 * phase-2 memory budget): when a feed would pass that size, Phase 1 runs on
 * the chunk fed so far and its superkmer records go, by bucket (a run of
 * consecutive minimizer bins, tg_job_opts.gpu_parts of them, 64 by default),
 * to host memory (dir == NULL) or to two files per bucket under dir. A
 * sequence-stream feed longer than a chunk is cut at a byte that separates
 * runs, a FASTA file before a record's '>'; a FASTQ file, or a single run or
 * record longer than a chunk, goes whole. tg_job_run then counts in passes over
 * consecutive buckets that fit the memory budget, uploading each pass's records
 * and keeping the pairs in host memory (results then stay on the host). The
 * pairs are the same as without spill. Call before the first feed; a job in
 * spill mode counts one sample, unsharded, and exports no partitions.
 * tg_stats.record_bytes receives the bytes spilled. */
tg_status tg_job_set_spill(tg_job* job, uint64_t chunk_bytes, const char* dir);

/* ---- shards: one job's partitions spread over devices ---------------------
 * Every instance of a canonical k-mer has the same minimizer, so the same bin
 * (partition): the pairs of different bins are disjoint. A job set to shard s
 * of n runs Phase 1 over its whole input and Phase 2 over the s-th of n equal
 * runs of consecutive bins only; its result is that shard's pairs, and the n
 * shards' results together are exactly the job's result. Device d of n counting
 * shard d of the same input is the partition -> device map of a multi-device
 * job, with no exchange between devices. n is a power of two, at most
 * TG_MAX_SHARDS (and at most tg_job_opts.gpu_parts when that is set); a job of
 * several samples cannot be sharded (TG_ERR_UNSUPPORTED from tg_job_run).
 * Call before tg_job_run. tg_stats.kmers, superkmers and bases describe the
 * whole input; distinct and out the shard. */
#define TG_MAX_SHARDS 1024u
tg_status tg_job_set_shard(tg_job* job, uint32_t shard, uint32_t n_shards);

/* ---- one-call helpers --------------------------------------------------- */
/* Count a host sequence stream end to end: H2D, both phases, D2H of the
 * filtered pairs into caller buffers of capacity cap (n_out receives the
 * number of pairs; TG_ERR_ARG if cap is too small, with n_out set). */
tg_status tg_count_seq(tg_ctx* ctx, const tg_job_opts* opts, const uint8_t* seq, size_t len,
                       uint64_t* keys, uint32_t* counts, uint64_t cap, uint64_t* n_out,
                       tg_stats* stats);
/* The same from the bytes of a FASTA/FASTQ file in host memory (pinned for
 * full-speed copies): H2D, lexing on the device, both phases, D2H. Replaces
 * SeqSource + run_callback (src/seq_source.hpp:190-205, src/pipeline.hpp:273-330). */
tg_status tg_count_fastx(tg_ctx* ctx, const tg_job_opts* opts, const uint8_t* data, size_t len,
                         uint64_t* keys, uint32_t* counts, uint64_t cap, uint64_t* n_out,
                         tg_stats* stats);
/* The same from the bytes of n_samples FASTA/FASTQ files in host memory, each
 * lexed on the device into its own sample (an empty one gives no pairs). */
tg_status tg_count_batch_fastx(tg_ctx* ctx, const tg_job_opts* opts, uint32_t n_samples,
                               const uint8_t* const* datas, const size_t* lens, uint64_t* keys,
                               uint32_t* counts, uint64_t* sample_offsets, uint64_t cap, uint64_t* n_out,
                               tg_stats* stats);
/* FASTA/FASTQ bytes to the sequence stream on the device, copied back to out
 * (capacity cap; *out_len receives the stream length, TG_ERR_ARG if it does not
 * fit). The stream holds the reference parser's ACGT runs in order, separated
 * by non-ACGT bytes. Needs a context with no active job. Replaces the
 * helicase parser (include/helicase_cpp/) as a stand-alone step. */
tg_status tg_fastx_to_stream(tg_ctx* ctx, const uint8_t* data, size_t len, uint8_t* out, size_t cap,
                             size_t* out_len);
/* The same for n_samples host sequence streams counted as separate samples in
 * one job: the pairs come back sample-major, sample i's being
 * [sample_offsets[i], sample_offsets[i+1]) (n_samples + 1 entries, may be NULL).
 * A batch larger than the device budget (hbm_budget_bytes, else free memory)
 * is counted as consecutive runs of whole samples, each run a job whose result
 * copy overlaps the next run; the call returns as one: the same offsets and
 * pairs, stats summed over the runs. With too small a cap, *n_out still
 * receives the total, TG_ERR_ARG is returned, and the samples that end within
 * cap are complete in keys/counts. */
tg_status tg_count_batch(tg_ctx* ctx, const tg_job_opts* opts, uint32_t n_samples,
                         const uint8_t* const* seqs, const size_t* lens, uint64_t* keys,
                         uint32_t* counts, uint64_t* sample_offsets, uint64_t cap, uint64_t* n_out,
                         tg_stats* stats);

/* Reads one input file into out (capacity cap; *out_len receives its length,
 * TG_ERR_ARG if it does not fit) exactly as tg_job_feed_file reads it: plain,
 * or inflated when the name ends in ".gz" (SeqSource's choice,
 * src/seq_source.hpp:196-204). BGZF files, whose members carry their sizes, are
 * inflated on `threads` host threads (0 = all cores); any other gzip file as
 * one stream, as the reference's GzInput (src/seq_source.hpp:48-141). Host
 * work only; errbuf (may be NULL) receives the message of a failure. */
tg_status tg_read_input(const char* path, uint32_t threads, uint8_t* out, size_t cap, size_t* out_len,
                        char* errbuf, size_t errlen);

/* ---- host memory for the host link --------------------------------------
 * No counterpart in the reference (its input never leaves host memory).
 * Page-locked host memory for the inputs and outputs of the one-call entry
 * points (tg_count_seq, tg_count_fastx, tg_count_batch*), from the CUDA
 * driver (portable to every device), so that a caller of this C ABI needs no
 * CUDA runtime of its own. Copies from and to it run at the host link's rate
 * (on a GB300: ~211 GB/s H2D, ~193 GB/s D2H); pageable memory goes through
 * staging copies. tg_host_free takes only pointers from tg_host_alloc
 * (TG_ERR_ARG otherwise). */
tg_status tg_host_alloc(size_t bytes, void** out);
tg_status tg_host_free(void* p);

/* ---- counting without device allocation --------------------------------
 * No counterpart in the reference: tuna allocates its partition buffers and
 * tables as it goes. This entry point is for callers that must not allocate
 * device memory when they call in: a plugin or inference-server enqueue that is
 * given a stream and its buffers, a process whose device memory belongs to
 * another allocator, or a loop where an allocation would stall the device.
 *
 * It counts a sequence stream already in device memory (d_seq, len bytes, the
 * convention of tg_job_feed_seq) and writes the pairs that pass ci/cx to the
 * caller's device buffers d_keys (cap * key words u64, see tg_job_key_words)
 * and d_counts (cap u32); *n_out receives the number of pairs. All work is
 * ordered on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 * the call returns when the result is complete. No cudaMalloc / cudaFree (or
 * any allocating library routine) is called: every intermediate array lives in
 * one device array of TG_NOALLOC_SCRATCH_BYTES in the library, which each GPU
 * that loads the library keeps reserved until the process exits.
 *   - len above TG_NOALLOC_MAX_LEN, or an input whose intermediate arrays do not
 *     fit in the scratch array, fails with TG_ERR_ARG and a message in errbuf
 *     (errbuf / errlen may be NULL / 0); k must be <= 63.
 *   - The array is reserved on a device by the first call there: the CUDA
 *     runtime loads the library's module for this entry point, which holds the
 *     array, when the call first looks up the array's device address (with that
 *     device current), so that call does allocate device memory. Make a first
 *     call with len == 0 (it only reserves the array) on each device before the
 *     caller's own allocator takes the device's memory and before any stream
 *     capture; or set CUDA_MODULE_LOADING=EAGER to reserve it when the library
 *     is loaded. Later calls allocate nothing.
 *   - The call blocks the calling host thread twice while it runs: once after
 *     Phase 1, to size Phase 2 from the record counts, and at the end.
 *   - gpu_parts: 0 or a power of two up to 4096, as tg_job_begin.
 *   - All calls share the one scratch array, so calls whose work overlaps on the
 *     GPU (two host threads, or two streams without ordering) race; serialise
 *     them. Each call re-initialises the parts that must start at zero.
 *   - Output capacity too small: TG_ERR_ARG with *n_out set to the needed size.
 */
#define TG_NOALLOC_MAX_LEN (1u << 19)
#define TG_NOALLOC_SCRATCH_BYTES (64u << 20)
tg_status tg_count_seq_device_noalloc(const tg_job_opts* opts, const uint8_t* d_seq, size_t len,
                                      uint64_t* d_keys, uint32_t* d_counts, uint64_t cap,
                                      uint64_t* n_out, void* stream, char* errbuf, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
