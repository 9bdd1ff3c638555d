// tg_api.cu — the C ABI of libtuna_gpu.so (include/tuna_gpu.h): contexts,
// jobs, the device pipeline driver and result access.
//
// A job runs, on the context's stream:
//   k_pack      ASCII stream -> 2-bit codes + validity bits
//   (k_lex_*    FASTA/FASTQ bytes -> the stream, when fed as files)
//   k_cut_seq   minimizers, chain starts, forced splits -> record descriptors
//               per CTA, k-mer instances per bin (one host sync here)
//   k_scan_*    bin counts -> key offsets
//   k_plan      groups of whole bins per segment (a run of bins of one sample)
//   k_keys      every canonical k-mer key at its bin's cursor
//   k_count     per group: keys into a shared-memory table, ci/cx, compaction
//               (again for groups split by key hash)
//   k_fb_*      (rare) key ranges that overflowed shared memory, global tables
//   k_fmt*      (tg_job_drain / tg_job_write) pairs -> TSV / KFF / raw bytes
// The export of partition files runs the tile cut k_cut<true> instead, which
// also yields each record's exact minimizer position.
//
// Reference counterparts (paths relative to the reference project root): a
// job is run<k,m> / run_callback<k,m> (src/pipeline.hpp:64-264, :273-330) with
// the input of SeqSource::process (src/seq_source.hpp:190-205); tg_job_stats
// carries what the stderr lines report (src/pipeline.hpp:174-178); the drain
// and tg_job_write are write_counts / write_counts_kff (src/count.hpp:180-265,
// src/kff_output.hpp:42-57); tg_job_export_partitions writes the disk
// pipeline's hash_<p>.superkmers (src/pipeline.hpp:186-201,
// src/superkmer_io.hpp:154-172); the one-call entry points are count_to_raw
// (include/tuna/tuna.hpp:181-195); passes over ranges of bins take the place
// of the disk mode (src/pipeline.hpp:77-98, :186-263).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "host/tg_host.h"
#include "tg_internal.cuh"
#include "tg_launch.h"
#include "tuna_gpu.h"

using namespace tg;

namespace {

constexpr uint64_t FWD_SEED[4] = {0x3c8bfbb395c60474ULL, 0x3193c18562a02b4cULL, 0x295549f54be24456ULL,
                                  0x20323ed082572324ULL};  // A C T G (nt codes), include/nt_hash.hpp:26-31

inline uint64_t hrol(uint64_t x, int s) { s &= 63; return s ? (x << s) | (x >> (64 - s)) : x; }
inline uint64_t hror(uint64_t x, int s) { s &= 63; return s ? (x >> s) | (x << (64 - s)) : x; }

}  // namespace

HashTables tg::make_hash_tables(int m) {
    HashTables T;
    for (int b = 0; b < 4; ++b) {
        const int nt = b ^ (b >> 1);  // kache A0 C1 G2 T3 -> nt A0 C1 T2 G3
        T.FW[b] = FWD_SEED[nt];
        T.RV[b] = FWD_SEED[nt ^ 2];   // REV[b] = FWD[complement(b)], complement = b ^ 2
    }
    for (int o = 0; o < 4; ++o)
        for (int i = 0; i < 4; ++i) {
            T.CTF[o * 4 + i] = hrol(T.FW[o], m) ^ T.FW[i];
            T.CTR[o * 4 + i] = hror(T.RV[o], 1) ^ hrol(T.RV[i], m - 1);
        }
    for (int v = 0; v < 256; ++v) {
        uint64_t f = 0, r = 0;
        for (int j = 0; j < 4; ++j) {
            const int b = (v >> (6 - 2 * j)) & 3;
            f ^= hrol(T.FW[b], 3 - j);
            r ^= hrol(T.RV[b], j);
        }
        T.GF[v] = f;
        T.GR[v] = r;
    }
    return T;
}

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

uint32_t next_pow2_u32(uint64_t v) {
    uint32_t p = 1;
    while (p < v && p < (1u << 31)) p <<= 1;
    return p;
}

// Layout of the small device counter buffer ctx->misc (byte offsets).
constexpr size_t MISC_CUT_STATS = 0;    // u64[3]: k-mers, records, runs (k_cut)
constexpr size_t MISC_BASES = 24;       // u64: ACGT bases (k_pack)
constexpr size_t MISC_OVERFLOW = 32;    // u32: descriptor list overflow (k_cut)
constexpr size_t MISC_DIGEST = 64;      // u64[4]: result digest (tg_job_result_digest)
constexpr size_t MISC_NDESC = 256;      // u32[C]: descriptors per Phase-1 CTA
constexpr size_t MISC_BYTES = MISC_NDESC + 4 * 65536;

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Host memcpy of n bytes on up to `threads` threads, each taking at least
// min_share bytes; the calling thread copies the first share. A share whose
// thread cannot be started is copied by the caller, so no joinable thread is
// ever left behind by an exception.
void parallel_copy(void* dst, const void* src, size_t n, unsigned threads, size_t min_share) {
    const size_t most = std::max<size_t>(1, n / std::max<size_t>(1, min_share));
    const unsigned nt = (unsigned)std::max<size_t>(1, std::min<size_t>(std::max(1u, threads), most));
    const size_t per = (n + nt - 1) / nt;
    auto part = [dst, src, n, per](unsigned t) {
        const size_t a = std::min(n, (size_t)t * per), b = std::min(n, a + per);
        if (b > a) memcpy(static_cast<uint8_t*>(dst) + a, static_cast<const uint8_t*>(src) + a, b - a);
    };
    std::vector<std::thread> th;
    th.reserve(nt);
    for (unsigned t = 1; t < nt; ++t) {
        try {
            th.emplace_back(part, t);
        } catch (...) {
            part(t);
        }
    }
    part(0);
    for (auto& t : th) t.join();
}

}  // namespace

struct tg_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    int n_sm = 0;
    uint64_t hbm_budget = 0;  // tg_ctx_opts.hbm_budget_bytes
    uint32_t flags = 0;       // tg_ctx_opts.flags
    uint32_t tuned_pct[2] = {0, 0};  // TG_CTX_AUTOTUNE: group size chosen per key width (0: not yet)
    size_t smem_optin = 0;
    unsigned host_threads = 1;
    std::string err;
    DevBuf seq, packed, valid, desc, xdesc, hist, scratch, okeys, ocnt, osamp, samp, okeys2, ocnt2, osoff,
        misc, fbtab, tables, raw, lexs, fbuf, fscr, sp_desc, sp_bytes, sp_aux;
    uint8_t* fhost[2] = {nullptr, nullptr};  // pinned host buffers of the output drain
    size_t fhost_cap = 0;
    uint8_t* stage[2] = {nullptr, nullptr};  // pinned staging of copies to pageable host memory
    cudaEvent_t ev[12] = {};
    // results copied to the host while counting runs (tg_count_seq)
    cudaStream_t st_copy = nullptr;
    unsigned long long* wave_out = nullptr;  // mapped pinned host, OVERLAP_WORDS entries
    unsigned long long* wave_out_dev = nullptr;
    cudaEvent_t wave_ev[16] = {};
    // a batch in runs of samples (count_host): the last run's result copy on
    // st_copy, which the next run's sample-major scatter waits for
    cudaEvent_t ev_copied = nullptr;
    bool copy_pending = false;
    tg_job* active = nullptr;
    int prepared_m = -1;

    tg_status fail(tg_status s, const std::string& msg) {
        if (s == TG_ERR_CUDA || s == TG_ERR_OOM) (void)cudaGetLastError();
        err = msg;
        return s;
    }
    // A failed runtime call also leaves its error as the thread's "last error",
    // which the next launch check would read: reset it once reported, so the
    // context's next job starts clean (a device fault stays sticky regardless).
    tg_status cuda_fail(cudaError_t e, const char* what) {
        (void)cudaGetLastError();
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? TG_ERR_OOM : TG_ERR_CUDA;
    }
    cudaError_t ensure(DevBuf& b, size_t bytes) {
        if (bytes <= b.cap && b.p) return cudaSuccess;
        if (b.p) {
            if (st_copy) cudaStreamSynchronize(st_copy);  // a result copy may still read it
            cudaFree(b.p);
            b.p = nullptr;
            b.cap = 0;
        }
        const size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&b.p, want);
        if (e != cudaSuccess) { b.p = nullptr; (void)cudaGetLastError(); return e; }
        b.cap = want;
        return cudaSuccess;
    }
};

// Host store of spill mode (tg_job_set_spill): per bucket (a run of
// 2^20 / nb consecutive bins), its record stream (2-bit bases, four per byte,
// in the byte order of the packed u32 words; every chunk's part a multiple of
// 4 bytes) and its descriptors (start = 4 x byte position in the stream), in
// host memory or in two files per bucket under `dir`; the k-mers per bin of
// all chunks; the chunks' phase-1 totals.
struct SpillStore {
    uint32_t nb = 64;
    int shift = 14;  // bucket = bin >> shift
    std::string dir;
    std::vector<tgh::Bytes> bytes;
    std::vector<std::vector<uint64_t>> desc;
    std::vector<uint64_t> n_bytes, n_desc;
    std::vector<uint64_t> hist;
    uint64_t kmers = 0, records = 0, runs = 0, bases = 0, chunks = 0, spilled_bytes = 0;
    std::string path(uint32_t b, const char* what) const {
        return dir + "/tuna_spill_" + std::to_string(b) + "." + what;
    }
    ~SpillStore() {
        if (dir.empty()) return;
        for (uint32_t b = 0; b < nb; ++b) {
            std::remove(path(b, "bytes").c_str());
            std::remove(path(b, "desc").c_str());
        }
    }
};

struct tg_job {
    tg_ctx* ctx = nullptr;
    tg_job_opts o{};
    int W = 1;
    int w = 0;
    uint32_t L = 0;
    // input stream
    size_t n = 0;                  // bytes in ctx->seq (or the external buffer)
    const uint8_t* ext = nullptr;  // single device feed, used in place
    bool used_ctx_seq = false;
    bool ran = false;
    // layout of the last run
    uint32_t p1_bits = 0, n_cta = 0;
    uint64_t chunk = 0, desc_cap = 0, packed_words = 0;
    // results
    uint64_t n_out = 0;
    tg_stats st{};
    // optional: output ranges handed out as phase 2 finishes them
    const P2Overlap* overlap = nullptr;
    // several samples: the sample-major copy waits for this event (count_host)
    cudaEvent_t reorder_after = nullptr;
    // samples: sample i starts at stream position sample_start[i]
    std::vector<unsigned long long> sample_start{0};
    int lex_launches = 0;  // lexer kernels of the feeds
    // phase 2 in passes (memory budget): the pairs are in host memory, either
    // the caller's buffers (sink_*, the one-call entry points) or host_keys/_counts
    bool spilled = false;
    std::vector<uint64_t, tgh::NoInitAlloc<uint64_t>> host_keys;
    std::vector<uint32_t, tgh::NoInitAlloc<uint32_t>> host_counts;
    uint64_t* sink_keys = nullptr;
    uint32_t* sink_counts = nullptr;
    uint64_t sink_cap = 0;
    // phase 2 over shard `shard` of `n_shards` runs of consecutive segments only
    uint32_t shard = 0, n_shards = 1;
    // spill mode: phase 1 per chunk of at most spill_chunk stream bytes, records
    // to the host store, phase 2 in passes over buckets read back from it
    bool spill = false;
    uint64_t spill_chunk = 0;
    std::unique_ptr<SpillStore> store;
    const uint8_t* seq_ptr() const { return ext ? ext : ctx->seq.as<uint8_t>(); }
};

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return ctx->cuda_fail(e_, what); \
    } while (0)

// NVTX range over one library call on the host thread (a profiler's timeline
// shows tg_job_run, its phase marks, the lexer and the drain); header-only
// NVTX does nothing unless a tool is attached.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// Ends a job the library opened itself, however the call leaves.
struct JobEnd {
    tg_job* j;
    ~JobEnd() { tg_job_end(j); }
};

static void note_host_failure(tg_ctx* ctx, const char* what) noexcept {
    if (!ctx) return;
    try {
        ctx->err = std::string("host: ") + what;
    } catch (...) {
    }
}

// Host-side C++ failures below the C ABI (allocation, thread creation, an
// exception from a caller's sink) become a status and a message: no exception
// crosses the ABI.
template <typename F>
static tg_status guarded(tg_ctx* ctx, F&& body) noexcept {
    try {
        return body();
    } catch (const std::exception& x) {
        note_host_failure(ctx, x.what());
    } catch (...) {
        note_host_failure(ctx, "unknown exception");
    }
    return TG_ERR_OOM;
}

extern "C" {

const char* tg_version(void) { return "tuna-gb300 0.1 (sm_103a)"; }

int tg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

static tg_status tg_ctx_create_impl(const tg_ctx_opts* opts, tg_ctx** out) {
    if (!out) return TG_ERR_ARG;
    *out = nullptr;
    tg_ctx_opts o{};
    if (opts) o = *opts;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TG_ERR_CUDA;
    if (o.device < 0 || o.device >= ndev) return TG_ERR_ARG;
    tg_ctx* ctx = new tg_ctx();
    ctx->device = o.device;
    ctx->hbm_budget = o.hbm_budget_bytes;
    ctx->flags = o.flags;
    ctx->host_threads = o.host_threads ? o.host_threads : std::max(1u, std::thread::hardware_concurrency());
    cudaError_t e = cudaSetDevice(o.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, o.device);
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, o.device);
    ctx->smem_optin = (size_t)optin;
    for (int i = 0; i < 12 && e == cudaSuccess; ++i) e = cudaEventCreate(&ctx->ev[i]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->st_copy, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaHostAlloc(&ctx->wave_out, OVERLAP_WORDS * sizeof(unsigned long long), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->wave_out_dev), ctx->wave_out, 0);
    for (int i = 0; i < 16 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&ctx->wave_ev[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_copied, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        tg_ctx_destroy(ctx);  // whatever was created so far
        (void)cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? TG_ERR_OOM : TG_ERR_CUDA;
    }
    *out = ctx;
    return TG_OK;
}

tg_status tg_ctx_create(const tg_ctx_opts* opts, tg_ctx** out) {
    return guarded(nullptr, [&] { return tg_ctx_create_impl(opts, out); });
}

tg_status tg_ctx_destroy(tg_ctx* ctx) {
    if (!ctx) return TG_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    if (ctx->st_copy) cudaStreamSynchronize(ctx->st_copy);
    DevBuf* bufs[] = {&ctx->seq, &ctx->packed, &ctx->valid, &ctx->desc, &ctx->xdesc, &ctx->hist,
                      &ctx->scratch,
                      &ctx->okeys, &ctx->ocnt, &ctx->osamp, &ctx->samp, &ctx->okeys2, &ctx->ocnt2, &ctx->osoff, &ctx->misc, &ctx->fbtab, &ctx->tables,
                      &ctx->raw, &ctx->lexs, &ctx->fbuf, &ctx->fscr, &ctx->sp_desc, &ctx->sp_bytes, &ctx->sp_aux};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->wave_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->ev_copied) cudaEventDestroy(ctx->ev_copied);
    if (ctx->st_copy) cudaStreamDestroy(ctx->st_copy);
    if (ctx->wave_out) cudaFreeHost(ctx->wave_out);
    for (uint8_t* h : ctx->fhost) tgh::pinned_free(h);
    for (uint8_t* h : ctx->stage) tgh::pinned_free(h);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return TG_OK;
}

const char* tg_last_error(const tg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* tg_ctx_stream(const tg_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

static tg_status tg_job_begin_impl(tg_ctx* ctx, const tg_job_opts* opts, tg_job** out) {
    if (!ctx || !opts || !out) return TG_ERR_ARG;
    *out = nullptr;
    const tg_job_opts& o = *opts;
    if (o.k < 2 || o.k > 256) return ctx->fail(TG_ERR_ARG, "k-mer length must be in [2, 256]");
    if (o.m < 1 || o.m > 32) return ctx->fail(TG_ERR_ARG, "minimizer length must be in [1, 32]");
    if (o.m >= o.k) return ctx->fail(TG_ERR_ARG, "minimizer length must be strictly less than k-mer length");
    if (o.k > 63) return ctx->fail(TG_ERR_UNSUPPORTED, "this GPU path supports k <= 63");
    if (o.n_parts & (o.n_parts - 1)) return ctx->fail(TG_ERR_ARG, "n_parts must be a power of two");
    if (o.gpu_parts & (o.gpu_parts - 1)) return ctx->fail(TG_ERR_ARG, "gpu_parts must be a power of two");
    if (o.gpu_parts > P1_MAX) return ctx->fail(TG_ERR_ARG, "gpu_parts must be <= 4096");
    if (ctx->active) return ctx->fail(TG_ERR_STATE, "another job is active on this context");
    tg_job* j = new tg_job();
    j->ctx = ctx;
    j->o = o;
    if (j->o.n_parts == 0) j->o.n_parts = 16;
    j->W = o.k <= 31 ? 1 : 2;
    j->w = o.k - o.m;
    const uint32_t hdr_max = (2u * o.k - o.m <= 255u) ? 255u : 65535u;
    j->L = hdr_max + 1 - o.k;
    ctx->active = j;
    *out = j;
    return TG_OK;
}

tg_status tg_job_begin(tg_ctx* ctx, const tg_job_opts* opts, tg_job** out) {
    return guarded(ctx, [&] { return tg_job_begin_impl(ctx, opts, out); });
}

// Room for `extra` more stream bytes in ctx->seq (a device feed used in place
// is moved into it first); *at receives the device address of position j->n.
static tg_status spill_flush(tg_job* j);

static tg_status stream_reserve(tg_job* j, size_t extra, uint8_t** at) {
    tg_ctx* ctx = j->ctx;
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (j->spill && j->n && j->n + extra > j->spill_chunk) {  // spill mode: this chunk is full
        const tg_status s = spill_flush(j);
        if (s != TG_OK) return s;
    }
    if (j->ext) {
        CK(ctx->ensure(ctx->seq, j->n + extra + 2), "alloc seq");
        CK(cudaMemcpyAsync(ctx->seq.p, j->ext, j->n, cudaMemcpyDeviceToDevice, ctx->st), "copy seq");
        j->ext = nullptr;
        j->used_ctx_seq = true;
    }
    const size_t need = j->n + extra + 1;
    if (need > ctx->seq.cap) {
        DevBuf nb;
        CK(cudaMalloc(&nb.p, std::max(need, 2 * ctx->seq.cap)), "alloc seq");
        nb.cap = std::max(need, 2 * ctx->seq.cap);
        if (j->n) CK(cudaMemcpyAsync(nb.p, ctx->seq.p, j->n, cudaMemcpyDeviceToDevice, ctx->st), "grow seq");
        CK(cudaStreamSynchronize(ctx->st), "grow seq");
        if (ctx->seq.p) cudaFree(ctx->seq.p);
        ctx->seq = nb;
    }
    *at = ctx->seq.as<uint8_t>() + j->n;
    return TG_OK;
}

static tg_status append_stream(tg_job* j, const uint8_t* src, size_t len, cudaMemcpyKind kind) {
    tg_ctx* ctx = j->ctx;
    if (j->ran) return ctx->fail(TG_ERR_STATE, "feed after run");
    uint8_t* d = nullptr;
    const tg_status s = stream_reserve(j, len + 1, &d);
    if (s != TG_OK) return s;
    const double t0 = now_ms();
    if (len) CK(link_copy(d, src, len, kind, ctx->st, ctx->n_sm), "copy input");
    CK(cudaMemsetAsync(d + len, '\n', 1, ctx->st), "separator");
    CK(cudaStreamSynchronize(ctx->st), "copy input");
    if (kind == cudaMemcpyHostToDevice) j->st.h2d_ms += now_ms() - t0;
    j->n += len + 1;
    j->used_ctx_seq = true;
    j->st.input_bytes += len;
    return TG_OK;
}

// FASTA/FASTQ bytes in device memory (16-byte aligned) lexed on the device
// onto the end of the stream. host_raw, when given, is the same bytes in host
// memory. A FASTQ file the device lexer flags (an empty header line at file
// offset 63 mod 64, where the reference's block walk departs from line
// counting) is parsed by the host parser instead.
static tg_status lex_append(tg_job* j, const uint8_t* draw, size_t len, const uint8_t* host_raw) {
    const TraceRange tr("tuna.lex");
    tg_ctx* ctx = j->ctx;
    if (j->ran) return ctx->fail(TG_ERR_STATE, "feed after run");
    if (len == 0) return ctx->fail(TG_ERR_PARSE, "Empty file");
    uint8_t* at = nullptr;
    tg_status s = stream_reserve(j, len + 1, &at);
    if (s != TG_OK) return s;
    uint8_t first = 0;
    if (host_raw) {
        first = host_raw[0];
    } else {
        CK(cudaMemcpyAsync(&first, draw, 1, cudaMemcpyDeviceToHost, ctx->st), "d2h");
        CK(cudaStreamSynchronize(ctx->st), "d2h");
    }
    const bool fastq = first == '@';
    CK(ctx->ensure(ctx->lexs, lex_scratch_bytes(len)), "alloc lexer scratch");
    LexTotals* dt = nullptr;
    int launches = 0;
    CK(cudaEventRecord(ctx->ev[10], ctx->st), "event");
    CK(launch_lex(draw, len, fastq, at, ctx->lexs.p, ctx->n_sm, ctx->st, &dt, &launches), "k_lex");
    CK(cudaEventRecord(ctx->ev[11], ctx->st), "event");
    LexTotals t{};
    CK(cudaMemcpyAsync(&t, dt, sizeof t, cudaMemcpyDeviceToHost, ctx->st), "d2h");
    CK(cudaStreamSynchronize(ctx->st), "k_lex");
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[10], ctx->ev[11]);
    j->st.lex_ms += ms;
    j->st.fastx_bytes += len;
    j->lex_launches += launches;
    if (t.irregular & 2u) return ctx->fail(TG_ERR_DEVICE, "FASTA/FASTQ lexer: a staging copy did not complete");
    if (t.irregular) {
        std::vector<uint8_t> hraw;
        if (!host_raw) {
            hraw.resize(len);
            CK(cudaMemcpy(hraw.data(), draw, len, cudaMemcpyDeviceToHost), "d2h");
            host_raw = hraw.data();
        }
        std::vector<uint8_t> st;
        tgh::fastx_to_stream(host_raw, len, st);
        j->st.host_parsed_bytes += len;
        return append_stream(j, st.data(), st.size(), cudaMemcpyHostToDevice);
    }
    CK(cudaMemsetAsync(at + t.out, '\n', 1, ctx->st), "separator");
    j->n += t.out + 1;
    j->used_ctx_seq = true;
    j->st.input_bytes += t.out;
    return TG_OK;
}

// Host FASTA/FASTQ bytes: copied to the device, lexed there.
static tg_status lex_append_host(tg_job* j, const uint8_t* data, size_t len) {
    tg_ctx* ctx = j->ctx;
    if (j->ran) return ctx->fail(TG_ERR_STATE, "feed after run");
    if (len == 0) return ctx->fail(TG_ERR_PARSE, "Empty file");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(ctx->ensure(ctx->raw, len + 16), "alloc raw input");
    const double t0 = now_ms();
    CK(link_copy(ctx->raw.p, data, len, cudaMemcpyHostToDevice, ctx->st, ctx->n_sm), "copy input");
    CK(cudaStreamSynchronize(ctx->st), "copy input");
    j->st.h2d_ms += now_ms() - t0;
    return lex_append(j, ctx->raw.as<uint8_t>(), len, data);
}

static inline bool is_acgt_byte(uint8_t c) {
    const uint8_t u = c & 0xDF;
    return u == 'A' || u == 'C' || u == 'G' || u == 'T';
}

static tg_status tg_job_feed_seq_impl(tg_job* j, const uint8_t* seq, size_t len) {
    if (!j || (!seq && len)) return TG_ERR_ARG;
    // spill mode: a feed longer than a chunk goes in pieces cut at a byte that
    // separates runs (nothing changes: every feed ends with a separator)
    while (j->spill && len > j->spill_chunk) {
        size_t cut = (size_t)j->spill_chunk;
        while (cut > 0 && is_acgt_byte(seq[cut])) --cut;
        if (cut == 0) break;  // one run longer than a chunk: fed whole
        const tg_status s = append_stream(j, seq, cut, cudaMemcpyHostToDevice);
        if (s != TG_OK) return s;
        seq += cut + 1;
        len -= cut + 1;
    }
    return append_stream(j, seq, len, cudaMemcpyHostToDevice);
}

tg_status tg_job_feed_seq(tg_job* j, const uint8_t* seq, size_t len) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_feed_seq_impl(j, seq, len); });
}

static tg_status tg_job_feed_seq_device_impl(tg_job* j, const uint8_t* dseq, size_t len) {
    if (!j || (!dseq && len)) return TG_ERR_ARG;
    if (j->ran) return j->ctx->fail(TG_ERR_STATE, "feed after run");
    if (j->n == 0 && !j->used_ctx_seq) {
        j->ext = dseq;
        j->n = len;
        j->st.input_bytes += len;
        return TG_OK;
    }
    return append_stream(j, dseq, len, cudaMemcpyDeviceToDevice);
}

tg_status tg_job_feed_seq_device(tg_job* j, const uint8_t* dseq, size_t len) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_feed_seq_device_impl(j, dseq, len); });
}

static tg_status tg_job_next_sample_impl(tg_job* j) {
    if (!j) return TG_ERR_ARG;
    if (j->ran) return j->ctx->fail(TG_ERR_STATE, "feed after run");
    if (j->sample_start.size() >= TG_MAX_SAMPLES) return j->ctx->fail(TG_ERR_ARG, "too many samples in one job");
    if (j->ext) {  // a device feed used in place: move it into the context buffer first
        const tg_status s = append_stream(j, nullptr, 0, cudaMemcpyDeviceToDevice);
        if (s != TG_OK) return s;
    }
    j->sample_start.push_back(j->n);
    return TG_OK;
}

tg_status tg_job_next_sample(tg_job* j) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_next_sample_impl(j); });
}

uint32_t tg_job_sample_count(const tg_job* j) { return j ? (uint32_t)j->sample_start.size() : 0; }

tg_status tg_job_set_shard(tg_job* j, uint32_t shard, uint32_t n_shards) {
    if (!j) return TG_ERR_ARG;
    if (j->ran) return j->ctx->fail(TG_ERR_STATE, "shard set after run");
    if (!n_shards || (n_shards & (n_shards - 1)) || n_shards > TG_MAX_SHARDS)
        return j->ctx->fail(TG_ERR_ARG, "n_shards must be a power of two <= 1024");
    if (shard >= n_shards) return j->ctx->fail(TG_ERR_ARG, "shard must be < n_shards");
    if (j->o.gpu_parts && j->o.gpu_parts < n_shards)
        return j->ctx->fail(TG_ERR_ARG, "n_shards must be <= gpu_parts");
    j->shard = shard;
    j->n_shards = n_shards;
    return TG_OK;
}

// Spill mode: a FASTA file longer than a chunk goes in pieces cut before a
// record's '>' (the parser restarts at every '>', so the runs are the same);
// FASTQ files go whole.
static tg_status feed_fastx_pieces(tg_job* j, const uint8_t* data, size_t len) {
    while (j->spill && len > j->spill_chunk && data[0] == '>') {
        size_t cut = (size_t)j->spill_chunk;
        while (cut > 1 && !(data[cut] == '>' && data[cut - 1] == '\n')) --cut;
        if (cut <= 1) break;  // one record longer than a chunk: fed whole
        const tg_status s = lex_append_host(j, data, cut);
        if (s != TG_OK) return s;
        data += cut;
        len -= cut;
    }
    return lex_append_host(j, data, len);
}

static tg_status tg_job_feed_fastx_impl(tg_job* j, const uint8_t* data, size_t len) {
    if (!j || (!data && len)) return TG_ERR_ARG;
    return feed_fastx_pieces(j, data, len);
}

tg_status tg_job_feed_fastx(tg_job* j, const uint8_t* data, size_t len) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_feed_fastx_impl(j, data, len); });
}

static tg_status tg_job_feed_fastx_device_impl(tg_job* j, const uint8_t* ddata, size_t len) {
    if (!j || (!ddata && len)) return TG_ERR_ARG;
    tg_ctx* ctx = j->ctx;
    if (j->ran) return ctx->fail(TG_ERR_STATE, "feed after run");
    if (len == 0) return ctx->fail(TG_ERR_PARSE, "Empty file");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (reinterpret_cast<uintptr_t>(ddata) & 15u) {  // the lexer loads 16-byte words
        CK(ctx->ensure(ctx->raw, len + 16), "alloc raw input");
        CK(cudaMemcpyAsync(ctx->raw.p, ddata, len, cudaMemcpyDeviceToDevice, ctx->st), "copy input");
        ddata = ctx->raw.as<uint8_t>();
    }
    return lex_append(j, ddata, len, nullptr);
}

tg_status tg_job_feed_fastx_device(tg_job* j, const uint8_t* ddata, size_t len) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_feed_fastx_device_impl(j, ddata, len); });
}

static tg_status tg_job_feed_file_impl(tg_job* j, const char* path) {
    if (!j || !path) return TG_ERR_ARG;
    tgh::Bytes raw;
    const std::string err = tgh::read_input_file(path, raw, j->ctx->host_threads);
    if (!err.empty()) {
        const bool empty = err.rfind("Empty file", 0) == 0;
        return j->ctx->fail(empty ? TG_ERR_PARSE : TG_ERR_IO, err);
    }
    return feed_fastx_pieces(j, raw.data(), raw.size());
}

tg_status tg_job_feed_file(tg_job* j, const char* path) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_feed_file_impl(j, path); });
}

static tg_status tg_read_input_impl(const char* path, uint32_t threads, uint8_t* out, size_t cap, size_t* out_len,
                        char* errbuf, size_t errlen) {
    if (!path || !out_len) return TG_ERR_ARG;
    *out_len = 0;
    auto set_err = [&](const std::string& m) {
        if (errbuf && errlen) {
            const size_t n = std::min(errlen - 1, m.size());
            memcpy(errbuf, m.data(), n);
            errbuf[n] = 0;
        }
    };
    tgh::Bytes raw;
    const std::string err =
        tgh::read_input_file(path, raw, threads ? threads : std::max(1u, std::thread::hardware_concurrency()));
    if (!err.empty()) {
        set_err(err);
        return err.rfind("Empty file", 0) == 0 ? TG_ERR_PARSE : TG_ERR_IO;
    }
    *out_len = raw.size();
    if (raw.size() > cap) {
        set_err("output buffer too small");
        return TG_ERR_ARG;
    }
    // the copy out, on the same threads for large files
    parallel_copy(out, raw.data(), raw.size(), threads ? threads : std::max(1u, std::thread::hardware_concurrency()),
                  16u << 20);
    return TG_OK;
}

tg_status tg_read_input(const char* path, uint32_t threads, uint8_t* out, size_t cap, size_t* out_len,
                        char* errbuf, size_t errlen) {
    try {
        return tg_read_input_impl(path, threads, out, cap, out_len, errbuf, errlen);
    } catch (const std::exception& x) {
        if (errbuf && errlen) snprintf(errbuf, errlen, "host: %s", x.what());
    } catch (...) {
        if (errbuf && errlen) snprintf(errbuf, errlen, "host: unknown exception");
    }
    return TG_ERR_OOM;
}

static tg_status tg_fastx_to_stream_impl(tg_ctx* ctx, const uint8_t* data, size_t len, uint8_t* out, size_t cap,
                             size_t* out_len) {
    if (!ctx || (!data && len) || !out_len) return TG_ERR_ARG;
    *out_len = 0;
    tg_job_opts o{};
    o.k = 31;
    o.m = 21;
    tg_job* j = nullptr;
    tg_status s = tg_job_begin(ctx, &o, &j);
    if (s != TG_OK) return s;
    const JobEnd end_job{j};
    s = tg_job_feed_fastx(j, data, len);
    if (s == TG_OK) {
        const size_t n = j->n ? j->n - 1 : 0;  // without the closing separator
        *out_len = n;
        if (n > cap) s = ctx->fail(TG_ERR_ARG, "stream buffer too small");
        else if (n) {
            cudaError_t e = cudaMemcpy(out, ctx->seq.p, n, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) s = ctx->cuda_fail(e, "d2h");
        }
    }
    return s;
}

tg_status tg_fastx_to_stream(tg_ctx* ctx, const uint8_t* data, size_t len, uint8_t* out, size_t cap,
                             size_t* out_len) {
    return guarded(ctx, [&] { return tg_fastx_to_stream_impl(ctx, data, len, out, cap, out_len); });
}

// Phase 1 cut (optionally the export variant) over the current stream.
struct CutSamples {
    const unsigned long long* start = nullptr;  // device arrays of the bin layout (counting cut)
    const uint32_t* base = nullptr;
    const uint8_t* bits = nullptr;
    uint32_t n = 0;
};

static tg_status run_cut(tg_job* j, bool exp, uint32_t p1_bits, int* launches, const CutSamples& cs = CutSamples()) {
    tg_ctx* ctx = j->ctx;
    const uint64_t n = j->n;
    const uint32_t p1 = 1u << p1_bits;
    const size_t smem = cut_smem_bytes(j->w, j->o.k, p1, exp);
    if (smem > ctx->smem_optin) return ctx->fail(TG_ERR_UNSUPPORTED, "phase-1 tile does not fit in shared memory");
    const uint64_t tile = cut_tile(j->w, exp);
    uint32_t C = (uint32_t)ctx->n_sm * cut_ctas_per_sm(j->w, j->o.k, p1, exp);
    uint64_t chunk = (n + C - 1) / C;
    chunk = std::max<uint64_t>(tile, (chunk + tile - 1) / tile * tile);
    C = (uint32_t)std::max<uint64_t>(1, (n + chunk - 1) / chunk);
    j->n_cta = C;
    j->chunk = chunk;
    j->p1_bits = p1_bits;
    // descriptors: about 2/(w+2) records per k-mer for random minimizers; grow on overflow
    double factor = std::min(1.0, 3.0 / (j->w + 2));
    for (int attempt = 0; attempt < 2; ++attempt) {
        const uint64_t cap = (uint64_t)(chunk * factor) + 2ull * tile + j->L + 64;
        j->desc_cap = cap;
        CK(ctx->ensure(ctx->desc, (size_t)C * cap * 8), "alloc descriptors");
        if (exp) CK(ctx->ensure(ctx->xdesc, (size_t)C * cap * 24), "alloc export descriptors");
        if (exp) {
            const size_t kmers_off = 4 * (size_t)hist_kmers_offset(p1, C);
            CK(ctx->ensure(ctx->hist, kmers_off + (size_t)p1 * 8), "alloc histograms");
            CK(cudaMemsetAsync(ctx->hist.as<uint8_t>() + kmers_off, 0, (size_t)p1 * 8, ctx->st), "memset");
        } else {
            CK(ctx->ensure(ctx->hist, (size_t)4 << BIN_BITS), "alloc bin histogram");
            CK(cudaMemsetAsync(ctx->hist.p, 0, (size_t)4 << BIN_BITS, ctx->st), "memset");
        }
        CK(cudaMemsetAsync(ctx->misc.as<uint8_t>() + MISC_CUT_STATS, 0, 24, ctx->st), "memset");
        CK(cudaMemsetAsync(ctx->misc.as<uint8_t>() + MISC_OVERFLOW, 0, 4, ctx->st), "memset");
        CutParams P{};
        P.packed = ctx->packed.as<uint32_t>();
        P.valid = ctx->valid.as<uint32_t>();
        P.n = n;
        P.k = j->o.k; P.m = j->o.m; P.w = j->w; P.L = j->L;
        P.p1_bits = p1_bits;
        P.n_cta = C;
        P.chunk = chunk;
        P.desc = ctx->desc.as<uint64_t>();
        P.desc_cap = cap;
        P.n_desc = reinterpret_cast<uint32_t*>(ctx->misc.as<uint8_t>() + MISC_NDESC);
        P.hist = exp ? ctx->hist.as<uint32_t>() : nullptr;
        P.binhist = exp ? nullptr : ctx->hist.as<uint32_t>();
        P.stats = reinterpret_cast<unsigned long long*>(ctx->misc.as<uint8_t>() + MISC_CUT_STATS);
        P.overflow = reinterpret_cast<uint32_t*>(ctx->misc.as<uint8_t>() + MISC_OVERFLOW);
        P.xdesc = exp ? ctx->xdesc.as<uint64_t>() : nullptr;
        P.sample_start = cs.start;
        P.sample_bin_base = cs.base;
        P.sample_bin_bits = cs.bits;
        P.n_samples = cs.n;
        CK(cudaEventRecord(ctx->ev[2], ctx->st), "event");
        CK(launch_cut(P, ctx->tables.as<HashTables>(), exp, ctx->st), "k_cut");
        CK(cudaEventRecord(ctx->ev[3], ctx->st), "event");
        ++*launches;
        uint32_t ovf = 0;
        CK(cudaMemcpyAsync(&ovf, ctx->misc.as<uint8_t>() + MISC_OVERFLOW, 4, cudaMemcpyDeviceToHost, ctx->st), "d2h");
        CK(cudaStreamSynchronize(ctx->st), "k_cut");
        if (!ovf) return TG_OK;
        factor = 1.0;  // every k-mer start can open a record at most once
    }
    return ctx->fail(TG_ERR_DEVICE, "descriptor capacity exceeded");
}

// Device memory to pageable host memory at the host link's rate: chunks are
// copied into the context's two pinned staging buffers in turn, and the host
// moves each one out with several threads while the next is copied.
static tg_status d2h_pageable(tg_ctx* ctx, void* dst, const void* src, size_t bytes) {
    constexpr size_t CH = 64u << 20;
    for (uint8_t*& b : ctx->stage)
        if (!b) {
            std::string why;
            b = static_cast<uint8_t*>(tgh::pinned_alloc(CH, &why));
            if (!b) return ctx->fail(TG_ERR_OOM, "pinned staging: " + why);
        }
    const size_t n_ch = (bytes + CH - 1) / CH;
    const unsigned nt = std::max(1u, std::min(ctx->host_threads, 16u));
    auto issue = [&](size_t c) -> cudaError_t {
        const size_t off = c * CH, len = std::min(CH, bytes - off);
        cudaError_t e = link_copy(ctx->stage[c & 1], static_cast<const uint8_t*>(src) + off, len,
                                  cudaMemcpyDeviceToHost, ctx->st, ctx->n_sm);
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[4 + (c & 1)], ctx->st);
        return e;
    };
    if (n_ch) CK(issue(0), "d2h");
    for (size_t c = 0; c < n_ch; ++c) {
        if (c + 1 < n_ch) CK(issue(c + 1), "d2h");  // the other buffer was emptied in the previous step
        CK(cudaEventSynchronize(ctx->ev[4 + (c & 1)]), "d2h");
        const size_t off = c * CH, len = std::min(CH, bytes - off);
        parallel_copy(static_cast<uint8_t*>(dst) + off, ctx->stage[c & 1], len, nt, 1u << 20);
    }
    return TG_OK;
}

// Phase 1 over the job's current stream: pack, then the cut into record
// descriptors (per-CTA lists) and the k-mers per bin. p1: segments of bins
// (0: chosen from the input size).
struct P1Out {
    SampleBins B;
    unsigned long long cstats[3] = {0, 0, 0};  // k-mers, records, runs
    unsigned long long n_bases = 0;
    std::vector<uint32_t> nd;                   // descriptors per list
};

static tg_status run_phase1(tg_job* j, int* launches_out, P1Out& r, uint32_t p1_force = 0) {
    tg_ctx* ctx = j->ctx;
    int launches = 0;
    const uint64_t n = j->n;
    if (n >= (1ull << DESC_START_BITS)) return ctx->fail(TG_ERR_ARG, "input stream longer than 2^36 bytes");
    // hash tables for m
    CK(ctx->ensure(ctx->tables, sizeof(HashTables)), "alloc tables");
    if (ctx->prepared_m != j->o.m) {
        const HashTables T = make_hash_tables(j->o.m);
        CK(cudaMemcpy(ctx->tables.p, &T, sizeof T, cudaMemcpyHostToDevice), "upload tables");
        ctx->prepared_m = j->o.m;
    }
    CK(ctx->ensure(ctx->misc, MISC_BYTES), "alloc misc");
    // ---- pack
    const uint64_t pw = packed_words_for(n);
    j->packed_words = pw;
    CK(ctx->ensure(ctx->packed, pw * 4), "alloc packed");
    CK(ctx->ensure(ctx->valid, (pw / 2) * 4 + 64), "alloc valid");
    CK(cudaMemsetAsync(ctx->misc.p, 0, MISC_NDESC, ctx->st), "memset");
    CK(cudaEventRecord(ctx->ev[0], ctx->st), "event");
    CK(launch_pack(j->seq_ptr(), n, ctx->packed.as<uint32_t>(), ctx->valid.as<uint32_t>(), pw,
                   reinterpret_cast<unsigned long long*>(ctx->misc.as<uint8_t>() + MISC_BASES), ctx->st), "k_pack");
    ++launches;
    CK(cudaEventRecord(ctx->ev[1], ctx->st), "event");
    CK(cudaMemcpyAsync(&r.n_bases, ctx->misc.as<uint8_t>() + MISC_BASES, 8, cudaMemcpyDeviceToHost, ctx->st), "d2h");
    // ---- phase 1: cut
    nvtxMarkA("tuna.phase1");
    uint32_t p1 = p1_force ? p1_force : j->o.gpu_parts;
    if (!p1) p1 = std::max(j->n_shards, std::min<uint32_t>(1024, std::max<uint32_t>(16, next_pow2_u32(n / 32768))));
    uint32_t p1_bits = 0;
    while ((1u << p1_bits) < p1) ++p1_bits;
    // the bins of the samples (2^20 in all, cut into p1 segments for one sample)
    std::vector<unsigned long long> starts = j->sample_start;
    starts.push_back(n);
    r.B = layout_bins(starts, (1u << BIN_BITS) >> p1_bits);
    const SampleBins& B = r.B;
    const uint32_t ns = (uint32_t)B.base.size();
    if (j->n_shards > 1 && ns > 1) return ctx->fail(TG_ERR_UNSUPPORTED, "a job of several samples cannot be sharded");
    {
        const size_t bytes = 8 * (size_t)(ns + 1) + 4 * (size_t)ns + ns + 64;
        CK(ctx->ensure(ctx->samp, bytes), "alloc samples");
        uint8_t* d = ctx->samp.as<uint8_t>();
        CK(cudaMemcpyAsync(d, B.start.data(), 8 * (size_t)(ns + 1), cudaMemcpyHostToDevice, ctx->st), "h2d");
        CK(cudaMemcpyAsync(d + 8 * (size_t)(ns + 1), B.base.data(), 4 * (size_t)ns, cudaMemcpyHostToDevice, ctx->st),
           "h2d");
        CK(cudaMemcpyAsync(d + 12 * (size_t)ns + 8, B.bits.data(), ns, cudaMemcpyHostToDevice, ctx->st), "h2d");
    }
    CutSamples cs;
    cs.start = ctx->samp.as<unsigned long long>();
    cs.base = reinterpret_cast<const uint32_t*>(ctx->samp.as<uint8_t>() + 8 * (size_t)(ns + 1));
    cs.bits = ctx->samp.as<uint8_t>() + 12 * (size_t)ns + 8;
    cs.n = ns;
    tg_status s = run_cut(j, false, p1_bits, &launches, cs);
    *launches_out += launches;
    if (s != TG_OK) return s;
    const uint32_t C = j->n_cta;
    r.nd.assign(C, 0);
    CK(cudaMemcpyAsync(r.cstats, ctx->misc.as<uint8_t>() + MISC_CUT_STATS, 24, cudaMemcpyDeviceToHost, ctx->st),
       "d2h");
    CK(cudaMemcpyAsync(r.nd.data(), ctx->misc.as<uint8_t>() + MISC_NDESC, (size_t)C * 4, cudaMemcpyDeviceToHost,
                       ctx->st), "d2h");
    CK(cudaStreamSynchronize(ctx->st), "phase 1");
    return TG_OK;
}

static tg_status run_spill(tg_job* j);

static tg_status tg_job_run_impl(tg_job* j) {
    if (!j) return TG_ERR_ARG;
    const TraceRange tr("tuna.job_run");
    tg_ctx* ctx = j->ctx;
    if (j->ran) return ctx->fail(TG_ERR_STATE, "job already ran");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (j->spill) return run_spill(j);
    int launches = 0;
    const int k = j->o.k;
    const int W = j->W;
    j->ran = true;
    P1Out r1;
    const tg_status s1 = run_phase1(j, &launches, r1);
    if (s1 != TG_OK) return s1;
    const SampleBins& B = r1.B;
    const uint32_t ns = (uint32_t)B.base.size();
    const unsigned long long* cstats = r1.cstats;
    const unsigned long long n_bases = r1.n_bases;
    const uint32_t C = j->n_cta;
    std::vector<uint32_t>& nd = r1.nd;
    nvtxMarkA("tuna.phase2");
    // ---- phase 2: one run over all bins or, when their keys and pairs do not
    // fit in the memory budget, passes over ranges of consecutive segments
    // (bins), each pass's pairs going to host memory before the next
    // the segments this run counts: all of them, or the job's shard of them
    std::vector<Segment> segs = B.segs;
    std::vector<uint32_t> hist;  // k-mers per bin, downloaded when a shard or the passes need it
    auto load_hist = [&]() -> cudaError_t {
        if (!hist.empty()) return cudaSuccess;
        hist.resize((size_t)1 << BIN_BITS);
        return cudaMemcpy(hist.data(), ctx->hist.p, hist.size() * 4, cudaMemcpyDeviceToHost);
    };
    uint64_t n_kmers = cstats[0];
    if (j->n_shards > 1) {  // one sample: 2^p1_bits >= n_shards segments of consecutive bins
        const size_t P = B.segs.size();
        segs.assign(B.segs.begin() + P * j->shard / j->n_shards, B.segs.begin() + P * (j->shard + 1) / j->n_shards);
        CK(load_hist(), "d2h");
        n_kmers = 0;
        for (const Segment& g : segs)
            for (uint32_t b = g.bin_lo; b < g.bin_hi; ++b) n_kmers += hist[b];
    }
    P2Input in{};
    in.W = W;
    in.k = k;
    in.segs = segs.data();
    in.n_segs = (uint32_t)segs.size();
    if (j->n_shards > 1) {
        in.bin_lo = segs.front().bin_lo;
        in.bin_hi = segs.back().bin_hi;
    }
    in.n_sm = (uint32_t)ctx->n_sm;
    in.packed = ctx->packed.as<uint32_t>();
    in.desc = ctx->desc.as<uint64_t>();
    in.desc_cap = j->desc_cap;
    in.n_lists = C;
    in.n_desc = nd.data();
    in.binhist = ctx->hist.as<uint32_t>();
    in.n_kmers = n_kmers;
    in.ci = j->o.ci;
    in.cx = j->o.cx;
    in.n_samples = ns;
    std::vector<std::pair<uint32_t, uint32_t>> passes;  // segment ranges
    std::vector<uint64_t> seg_keys;
    {
        const uint64_t per_key = 2 * key_bytes(W) + 4 + 24;  // key, pair, groups and slack
        size_t free_b = 0, total_b = 0;
        CK(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
        const uint64_t have = free_b + ctx->scratch.cap + ctx->okeys.cap + ctx->ocnt.cap;
        const uint64_t reserve = (2ull << 30) + total_b / 50;
        const uint64_t budget = ctx->hbm_budget ? ctx->hbm_budget : (have > reserve ? have - reserve : 0);
        if (ns == 1 && segs.size() > 1 && n_kmers * per_key > budget) {
            CK(load_hist(), "d2h");
            const uint64_t max_keys = std::max<uint64_t>(1, budget / per_key);
            uint32_t s0 = 0;
            uint64_t acc = 0;
            for (uint32_t sg = 0; sg < segs.size(); ++sg) {
                uint64_t kk = 0;
                for (uint32_t b = segs[sg].bin_lo; b < segs[sg].bin_hi; ++b) kk += hist[b];
                seg_keys.push_back(kk);
                if (sg > s0 && acc + kk > max_keys) {
                    passes.emplace_back(s0, sg);
                    s0 = sg;
                    acc = 0;
                }
                acc += kk;
            }
            passes.emplace_back(s0, (uint32_t)segs.size());
        }
    }
    CK(cudaEventRecord(ctx->ev[6], ctx->st), "event");
    std::string msg;
    auto fallback_table = [&](size_t bytes) -> void* {
        return ctx->ensure(ctx->fbtab, bytes) == cudaSuccess ? ctx->fbtab.p : nullptr;
    };
    P2Output out{};
    tg_stats& S = j->st;
    float ms = 0;
    if (passes.size() <= 1) {
        const uint64_t out_cap = std::max<uint64_t>(n_kmers, 1);
        CK(ctx->ensure(ctx->okeys, out_cap * key_bytes(W)), "alloc output keys");
        CK(ctx->ensure(ctx->ocnt, out_cap * 4), "alloc output counts");
        if (ns > 1) {
            CK(ctx->ensure(ctx->osamp, out_cap * 4), "alloc output samples");
            CK(ctx->ensure(ctx->okeys2, out_cap * key_bytes(W)), "alloc output keys");
            CK(ctx->ensure(ctx->ocnt2, out_cap * 4), "alloc output counts");
            CK(ctx->ensure(ctx->osoff, 8 * ((size_t)ns + 1)), "alloc sample offsets");
        }
        out.keys = ctx->okeys.p;
        out.counts = ctx->ocnt.as<uint32_t>();
        out.samples = ns > 1 ? ctx->osamp.as<uint32_t>() : nullptr;
        out.n_samples = ns;
        if (ns > 1) {
            out.keys2 = ctx->okeys2.p;
            out.counts2 = ctx->ocnt2.as<uint32_t>();
            out.sample_off = ctx->osoff.as<unsigned long long>();
            out.reorder_after = j->reorder_after;
        }
        out.cap = out_cap;
        // group size: the context's tuned one, else half the table; with
        // TG_CTX_AUTOTUNE the first large job of a key width times the counting
        // pass at each candidate on its own keys and keeps the fastest
        uint32_t pct = ctx->tuned_pct[W - 1] ? ctx->tuned_pct[W - 1] : 50;
        if ((ctx->flags & TG_CTX_AUTOTUNE) && !ctx->tuned_pct[W - 1] && n_kmers >= (1ull << 26)) {
            static const uint32_t cand[] = {35, 50, 65};
            float best = 0;
            for (uint32_t cp : cand) {
                P2Input ti = in;
                ti.group_pct = cp;
                const size_t tb = phase2_scratch_bytes(ti);
                CK(ctx->ensure(ctx->scratch, tb), "alloc phase-2 scratch");
                P2Output to = out;
                const tg_status ts = phase2_run(ti, ctx->scratch.p, tb, to, fallback_table, ctx->st, ctx->ev[7],
                                                &launches, msg, P2Overlap());
                if (ts != TG_OK) return ctx->fail(ts, msg);
                CK(cudaEventRecord(ctx->ev[8], ctx->st), "event");
                CK(cudaEventSynchronize(ctx->ev[8]), "sync");
                cudaEventElapsedTime(&ms, ctx->ev[7], ctx->ev[8]);  // the counting pass (keys come before ev[7])
                if (S.autotune_trials == 0 || ms < best) { best = ms; pct = cp; }
                ++S.autotune_trials;
            }
            ctx->tuned_pct[W - 1] = pct;
        }
        in.group_pct = pct;
        S.group_load_pct = pct;
        const size_t p2_bytes = phase2_scratch_bytes(in);
        CK(ctx->ensure(ctx->scratch, p2_bytes), "alloc phase-2 scratch");
        CK(cudaEventRecord(ctx->ev[6], ctx->st), "event");
        const tg_status ps = phase2_run(in, ctx->scratch.p, p2_bytes, out, fallback_table, ctx->st, ctx->ev[7],
                                        &launches, msg, j->overlap ? *j->overlap : P2Overlap());
        if (ps != TG_OK) return ctx->fail(ps, msg);
        CK(cudaEventRecord(ctx->ev[8], ctx->st), "event");
        CK(cudaEventSynchronize(ctx->ev[8]), "sync");
        j->n_out = out.n_out;
        S.distinct = out.distinct;
        S.fallback_groups = out.fallback_groups;
        S.groups = out.groups;
        S.heavy_groups = (uint32_t)out.heavy_groups;
        cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[8]); S.phase2_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]); S.phase2_keys_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev[7], ctx->ev[8]); S.phase2_count_ms = ms;
        S.phase2_passes = 1;
    } else {
        // sizes of the largest pass
        uint64_t max_keys = 0;
        in.group_pct = ctx->tuned_pct[W - 1] ? ctx->tuned_pct[W - 1] : 50;
        S.group_load_pct = in.group_pct;
        std::vector<P2Input> pin(passes.size(), in);
        size_t p2_bytes = 0;
        for (size_t p = 0; p < passes.size(); ++p) {
            P2Input& ip = pin[p];
            const uint32_t s0 = passes[p].first, s1 = passes[p].second;
            ip.segs = segs.data() + s0;
            ip.n_segs = s1 - s0;
            ip.bin_lo = segs[s0].bin_lo;
            ip.bin_hi = segs[s1 - 1].bin_hi;
            ip.n_kmers = 0;
            for (uint32_t sg = s0; sg < s1; ++sg) ip.n_kmers += seg_keys[sg];
            max_keys = std::max(max_keys, ip.n_kmers);
            p2_bytes = std::max(p2_bytes, phase2_scratch_bytes(ip));
        }
        const uint64_t out_cap = std::max<uint64_t>(max_keys, 1);
        CK(ctx->ensure(ctx->okeys, out_cap * key_bytes(W)), "alloc output keys");
        CK(ctx->ensure(ctx->ocnt, out_cap * 4), "alloc output counts");
        CK(ctx->ensure(ctx->scratch, p2_bytes), "alloc phase-2 scratch");
        j->spilled = true;
        j->host_keys.clear();
        j->host_counts.clear();
        if (!(j->sink_keys || j->sink_counts)) {  // at most one pair per k-mer: no reallocation between passes
            j->host_keys.reserve(n_kmers * W);
            j->host_counts.reserve(n_kmers);
        }
        uint64_t acc = 0;
        const double t0 = now_ms();
        for (size_t p = 0; p < passes.size(); ++p) {
            P2Output po{};
            po.keys = ctx->okeys.p;
            po.counts = ctx->ocnt.as<uint32_t>();
            po.cap = out_cap;
            CK(cudaEventRecord(ctx->ev[6], ctx->st), "event");
            const tg_status ps = phase2_run(pin[p], ctx->scratch.p, p2_bytes, po, fallback_table, ctx->st,
                                            ctx->ev[7], &launches, msg, P2Overlap());
            if (ps != TG_OK) return ctx->fail(ps, msg);
            CK(cudaEventRecord(ctx->ev[8], ctx->st), "event");
            CK(cudaEventSynchronize(ctx->ev[8]), "sync");
            cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]); S.phase2_keys_ms += ms;
            cudaEventElapsedTime(&ms, ctx->ev[7], ctx->ev[8]); S.phase2_count_ms += ms;
            const uint64_t n_p = po.n_out;
            const double c0 = now_ms();
            if (j->sink_keys || j->sink_counts) {  // straight into the caller's buffers, as far as they reach
                const uint64_t m = acc < j->sink_cap ? std::min(n_p, j->sink_cap - acc) : 0;
                if (m && j->sink_keys)
                    CK(link_copy(j->sink_keys + acc * W, po.keys, m * key_bytes(W), cudaMemcpyDeviceToHost, ctx->st,
                                 ctx->n_sm), "d2h");
                if (m && j->sink_counts)
                    CK(link_copy(j->sink_counts + acc, po.counts, m * 4, cudaMemcpyDeviceToHost, ctx->st, ctx->n_sm),
                       "d2h");
                CK(cudaStreamSynchronize(ctx->st), "d2h");
            } else if (n_p) {
                j->host_keys.resize((acc + n_p) * W);
                j->host_counts.resize(acc + n_p);
                tg_status cs = d2h_pageable(ctx, j->host_keys.data() + acc * W, po.keys, n_p * key_bytes(W));
                if (cs == TG_OK) cs = d2h_pageable(ctx, j->host_counts.data() + acc, po.counts, n_p * 4);
                if (cs != TG_OK) return cs;
            }
            S.d2h_ms += now_ms() - c0;
            acc += n_p;
            S.distinct += po.distinct;
            S.fallback_groups += po.fallback_groups;
            S.groups += po.groups;
            S.heavy_groups += (uint32_t)po.heavy_groups;
        }
        S.phase2_ms = now_ms() - t0;
        S.phase2_passes = passes.size();
        j->n_out = acc;
    }
    // ---- stats
    S.bases = n_bases;
    S.runs = cstats[2];
    S.kmers = cstats[0];
    S.superkmers = cstats[1];
    S.out = j->n_out;
    S.gpu_parts = (uint32_t)B.segs.size();
    S.record_bytes = cstats[1] * 8;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]); S.pack_ms = ms;
    cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]); S.phase1_cut_ms = ms;
    S.phase1_scatter_ms = 0;  // records stay in the cut's lists
    S.phase1_ms = S.phase1_cut_ms;
    S.gpu_launches = (uint64_t)(launches + j->lex_launches);
    return TG_OK;
}

tg_status tg_job_run(tg_job* j) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_run_impl(j); });
}

// ---------------------------------------------------------------- spill mode
// The device budget phase 2 may use (tg_ctx_opts.hbm_budget_bytes, else free
// memory plus the context's reusable buffers minus a reserve).
static tg_status phase2_budget(tg_ctx* ctx, uint64_t* budget) {
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    const uint64_t have = free_b + ctx->scratch.cap + ctx->okeys.cap + ctx->ocnt.cap;
    const uint64_t reserve = (2ull << 30) + total_b / 50;
    *budget = ctx->hbm_budget ? ctx->hbm_budget : (have > reserve ? have - reserve : 0);
    return TG_OK;
}

tg_status tg_job_set_spill(tg_job* j, uint64_t chunk_bytes, const char* dir) {
    if (!j) return TG_ERR_ARG;
    tg_ctx* ctx = j->ctx;
    return guarded(ctx, [&]() -> tg_status {
        if (j->ran || j->n || j->ext) return ctx->fail(TG_ERR_STATE, "spill mode is set before the first feed");
        if (j->sample_start.size() > 1 || j->n_shards > 1)
            return ctx->fail(TG_ERR_UNSUPPORTED, "spill mode counts one sample, unsharded");
        if (!chunk_bytes) {
            uint64_t budget = 0;
            const tg_status s = phase2_budget(ctx, &budget);
            if (s != TG_OK) return s;
            chunk_bytes = std::max<uint64_t>(1ull << 24, budget / 16);
        }
        auto st = std::make_unique<SpillStore>();
        st->nb = j->o.gpu_parts ? std::max<uint32_t>(16, std::min<uint32_t>(j->o.gpu_parts, SPILL_MAX_BUCKETS)) : 64;
        st->shift = BIN_BITS;
        for (uint32_t v = st->nb; v > 1; v >>= 1) --st->shift;
        st->dir = dir ? dir : "";
        st->bytes.resize(dir ? 0 : st->nb);
        st->desc.resize(dir ? 0 : st->nb);
        st->n_bytes.assign(st->nb, 0);
        st->n_desc.assign(st->nb, 0);
        st->hist.assign((size_t)1 << BIN_BITS, 0);
        if (dir) {  // fresh, empty bucket files
            for (uint32_t b = 0; b < st->nb; ++b)
                for (const char* what : {"bytes", "desc"}) {
                    FILE* f = std::fopen(st->path(b, what).c_str(), "wb");
                    if (!f) return ctx->fail(TG_ERR_IO, "cannot create spill file " + st->path(b, what));
                    std::fclose(f);
                }
        }
        j->store = std::move(st);
        j->spill = true;
        j->spill_chunk = chunk_bytes;
        return TG_OK;
    });
}

static tg_status append_file(tg_ctx* ctx, const std::string& path, const void* data, size_t bytes) {
    if (!bytes) return TG_OK;
    FILE* f = std::fopen(path.c_str(), "ab");
    if (!f) return ctx->fail(TG_ERR_IO, "cannot open spill file " + path);
    const size_t w = std::fwrite(data, 1, bytes, f);
    const bool ok = std::fclose(f) == 0 && w == bytes;
    return ok ? TG_OK : ctx->fail(TG_ERR_IO, "cannot write spill file " + path);
}

static tg_status read_file(tg_ctx* ctx, const std::string& path, void* out, size_t bytes) {
    if (!bytes) return TG_OK;
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return ctx->fail(TG_ERR_IO, "cannot open spill file " + path);
    const size_t r = std::fread(out, 1, bytes, f);
    std::fclose(f);
    return r == bytes ? TG_OK : ctx->fail(TG_ERR_IO, "short spill file " + path);
}

// Phase 1 of the chunk fed so far; its records to the store, by bucket.
static tg_status spill_flush(tg_job* j) {
    tg_ctx* ctx = j->ctx;
    SpillStore& S = *j->store;
    if (!j->n) return TG_OK;
    int launches = 0;
    P1Out r;
    tg_status s = run_phase1(j, &launches, r, S.nb);
    if (s != TG_OK) return s;
    const uint32_t nb = S.nb, C = j->n_cta;
    const uint32_t* d_nd = reinterpret_cast<const uint32_t*>(ctx->misc.as<uint8_t>() + MISC_NDESC);
    {  // k-mers per bin
        std::vector<uint32_t> h((size_t)1 << BIN_BITS);
        CK(cudaMemcpy(h.data(), ctx->hist.p, h.size() * 4, cudaMemcpyDeviceToHost), "d2h");
        for (size_t b = 0; b < h.size(); ++b) S.hist[b] += h[b];
    }
    // per-bucket records and bytes, then the staging layout
    // sp_aux: totals [2 nb], cursors [2 nb], host shifts [nb] (u64 / i64 each)
    CK(ctx->ensure(ctx->sp_aux, 8 * 5 * (size_t)nb), "alloc spill counters");
    unsigned long long* d_tot = ctx->sp_aux.as<unsigned long long>();
    CK(launch_spill_size(ctx->desc.as<uint64_t>(), j->desc_cap, d_nd, C, j->o.k, S.shift, nb, d_tot, ctx->st),
       "k_spill_size");
    std::vector<unsigned long long> tot(2 * (size_t)nb);
    CK(cudaMemcpyAsync(tot.data(), d_tot, 16 * (size_t)nb, cudaMemcpyDeviceToHost, ctx->st), "d2h");
    CK(cudaStreamSynchronize(ctx->st), "k_spill_size");
    std::vector<unsigned long long> cur(2 * (size_t)nb);
    std::vector<long long> shift(nb);
    uint64_t recs = 0, bytes = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        // a descriptor's start is 4 x the record's byte position in its bucket
        if (4 * (S.n_bytes[b] + tot[nb + b] + 4) >= (1ull << DESC_START_BITS))
            return ctx->fail(TG_ERR_UNSUPPORTED, "a spill bucket passes 2^34 bytes; use more buckets (gpu_parts)");
        cur[b] = recs;
        cur[nb + b] = bytes;
        shift[b] = (long long)S.n_bytes[b] - (long long)bytes;
        recs += tot[b];
        bytes += (tot[nb + b] + 3) & ~3ull;  // every bucket's part a multiple of 4 bytes
    }
    CK(ctx->ensure(ctx->sp_desc, recs * 8 + 8), "alloc spill descriptors");
    CK(ctx->ensure(ctx->sp_bytes, bytes + 16), "alloc spill bytes");
    CK(cudaMemsetAsync(ctx->sp_bytes.p, 0, bytes + 16, ctx->st), "memset");
    unsigned long long* d_cur = d_tot + 2 * (size_t)nb;
    long long* d_shift = reinterpret_cast<long long*>(d_tot + 4 * (size_t)nb);
    CK(cudaMemcpyAsync(d_cur, cur.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, ctx->st), "h2d");
    CK(cudaMemcpyAsync(d_shift, shift.data(), 8 * (size_t)nb, cudaMemcpyHostToDevice, ctx->st), "h2d");
    CK(launch_spill_write(ctx->packed.as<uint32_t>(), ctx->desc.as<uint64_t>(), j->desc_cap, d_nd, C, j->o.k,
                          S.shift, nb, d_cur, d_shift, ctx->sp_desc.as<uint64_t>(), ctx->sp_bytes.as<uint8_t>(),
                          ctx->st), "k_spill_write");
    launches += 2;
    j->lex_launches += launches;  // counted with the job's other launches
    // to the store
    std::vector<uint64_t> hd(recs);
    tgh::Bytes hb(bytes);
    s = d2h_pageable(ctx, hd.data(), ctx->sp_desc.p, recs * 8);
    if (s == TG_OK) s = d2h_pageable(ctx, hb.data(), ctx->sp_bytes.p, bytes);
    if (s != TG_OK) return s;
    for (uint32_t b = 0; b < nb; ++b) {
        const uint64_t r0 = cur[b], rn = tot[b];
        const uint64_t b0 = cur[nb + b], bn = (tot[nb + b] + 3) & ~3ull;
        if (S.dir.empty()) {
            S.desc[b].insert(S.desc[b].end(), hd.begin() + r0, hd.begin() + r0 + rn);
            S.bytes[b].insert(S.bytes[b].end(), hb.begin() + b0, hb.begin() + b0 + bn);
        } else {
            s = append_file(ctx, S.path(b, "desc"), hd.data() + r0, rn * 8);
            if (s == TG_OK) s = append_file(ctx, S.path(b, "bytes"), hb.data() + b0, bn);
            if (s != TG_OK) return s;
        }
        S.n_desc[b] += rn;
        S.n_bytes[b] += bn;
    }
    S.kmers += r.cstats[0];
    S.records += r.cstats[1];
    S.runs += r.cstats[2];
    S.bases += r.n_bases;
    S.spilled_bytes += recs * 8 + bytes;
    ++S.chunks;
    j->n = 0;
    j->ext = nullptr;
    return TG_OK;
}

// Phase 2 of a spill-mode job: passes over consecutive buckets whose keys and
// pairs fit the budget; each pass uploads its buckets' record streams (one
// after the other, each at a 16-base boundary after the leading pad) and
// descriptors (rebased to the pass stream) and counts them.
static tg_status run_spill(tg_job* j) {
    tg_ctx* ctx = j->ctx;
    SpillStore& S = *j->store;
    tg_status s = spill_flush(j);
    if (s != TG_OK) return s;
    j->ran = true;
    const int W = j->W, k = j->o.k;
    const uint32_t nb = S.nb;
    const uint32_t seg_bins = (1u << BIN_BITS) / nb;
    int launches = 0;
    // k-mers per bin of all chunks, for the scan of each pass
    std::vector<uint32_t> h32(S.hist.size());
    std::vector<uint64_t> bk(nb, 0);
    for (size_t b = 0; b < S.hist.size(); ++b) {
        if (S.hist[b] > 0xFFFFFFFFull) return ctx->fail(TG_ERR_UNSUPPORTED, "a bin holds more than 2^32 k-mers");
        h32[b] = (uint32_t)S.hist[b];
        bk[b / seg_bins] += S.hist[b];
    }
    CK(ctx->ensure(ctx->hist, (size_t)4 << BIN_BITS), "alloc bin histogram");
    CK(cudaMemcpy(ctx->hist.p, h32.data(), h32.size() * 4, cudaMemcpyHostToDevice), "h2d");
    const SampleBins B = layout_bins({0ull, 1ull}, seg_bins);
    uint64_t budget = 0;
    s = phase2_budget(ctx, &budget);
    if (s != TG_OK) return s;
    const uint64_t per_key = 2 * key_bytes(W) + 4 + 24;
    const uint64_t max_keys = std::max<uint64_t>(1, budget / per_key);
    std::vector<std::pair<uint32_t, uint32_t>> passes;
    for (uint32_t b0 = 0, b = 0; b <= nb; ++b) {
        uint64_t acc = 0, bytes = 0;
        for (uint32_t x = b0; x < b; ++x) { acc += bk[x]; bytes += S.n_bytes[x]; }
        const bool full = b < nb && b > b0 && (acc + bk[b] > max_keys || 4 * (bytes + S.n_bytes[b]) >= (1ull << 35));
        if (b == nb || full) {
            if (b > b0) passes.emplace_back(b0, b);
            b0 = b;
        }
    }
    tg_stats& T = j->st;
    T.group_load_pct = ctx->tuned_pct[W - 1] ? ctx->tuned_pct[W - 1] : 50;
    auto fallback_table = [&](size_t bytes) -> void* {
        return ctx->ensure(ctx->fbtab, bytes) == cudaSuccess ? ctx->fbtab.p : nullptr;
    };
    j->spilled = true;
    j->host_keys.clear();
    j->host_counts.clear();
    if (!(j->sink_keys || j->sink_counts)) {
        j->host_keys.reserve(S.kmers * W);
        j->host_counts.reserve(S.kmers);
    }
    std::string msg;
    uint64_t acc = 0;
    float ms = 0;
    const double t0 = now_ms();
    for (const auto& pr : passes) {
        uint64_t nbytes = 0, ndesc = 0, nk = 0;
        for (uint32_t b = pr.first; b < pr.second; ++b) { nbytes += S.n_bytes[b]; ndesc += S.n_desc[b]; nk += bk[b]; }
        if (ndesc > 0xFFFFFFFFull) return ctx->fail(TG_ERR_UNSUPPORTED, "a spill pass holds more than 2^32 records");
        // the pass stream: 8 bytes (TG_PAD bases) of padding, the buckets, slack
        const uint64_t words = packed_words_for(4 * nbytes);
        CK(ctx->ensure(ctx->packed, words * 4), "alloc packed");
        CK(cudaMemsetAsync(ctx->packed.p, 0, words * 4, ctx->st), "memset");
        CK(ctx->ensure(ctx->desc, ndesc * 8 + 8), "alloc descriptors");
        uint64_t bo = 0, dof = 0;
        for (uint32_t b = pr.first; b < pr.second; ++b) {
            uint8_t* dst_bytes = ctx->packed.as<uint8_t>() + 8 + bo;
            uint64_t* dst_desc = ctx->desc.as<uint64_t>() + dof;
            if (S.dir.empty()) {
                CK(cudaMemcpyAsync(dst_bytes, S.bytes[b].data(), S.n_bytes[b], cudaMemcpyHostToDevice, ctx->st), "h2d");
                CK(cudaMemcpyAsync(dst_desc, S.desc[b].data(), S.n_desc[b] * 8, cudaMemcpyHostToDevice, ctx->st),
                   "h2d");
            } else {
                tgh::Bytes tmp(S.n_bytes[b] + S.n_desc[b] * 8);
                s = read_file(ctx, S.path(b, "bytes"), tmp.data(), S.n_bytes[b]);
                if (s == TG_OK) s = read_file(ctx, S.path(b, "desc"), tmp.data() + S.n_bytes[b], S.n_desc[b] * 8);
                if (s != TG_OK) return s;
                CK(cudaMemcpyAsync(dst_bytes, tmp.data(), S.n_bytes[b], cudaMemcpyHostToDevice, ctx->st), "h2d");
                CK(cudaMemcpyAsync(dst_desc, tmp.data() + S.n_bytes[b], S.n_desc[b] * 8, cudaMemcpyHostToDevice,
                                   ctx->st), "h2d");
                CK(cudaStreamSynchronize(ctx->st), "h2d");
            }
            CK(launch_rebase(dst_desc, S.n_desc[b], 4 * bo, ctx->n_sm, ctx->st), "k_rebase");
            bo += S.n_bytes[b];
            dof += S.n_desc[b];
        }
        const uint32_t nlist = (uint32_t)ndesc;
        P2Input in{};
        in.W = W;
        in.k = k;
        in.segs = B.segs.data() + pr.first;
        in.n_segs = pr.second - pr.first;
        in.bin_lo = B.segs[pr.first].bin_lo;
        in.bin_hi = B.segs[pr.second - 1].bin_hi;
        in.n_sm = (uint32_t)ctx->n_sm;
        in.packed = ctx->packed.as<uint32_t>();
        in.desc = ctx->desc.as<uint64_t>();
        in.desc_cap = std::max<uint64_t>(ndesc, 1);
        in.n_lists = 1;
        in.n_desc = &nlist;
        in.binhist = ctx->hist.as<uint32_t>();
        in.n_kmers = nk;
        in.ci = j->o.ci;
        in.cx = j->o.cx;
        in.n_samples = 1;
        in.group_pct = T.group_load_pct;
        const uint64_t out_cap = std::max<uint64_t>(nk, 1);
        CK(ctx->ensure(ctx->okeys, out_cap * key_bytes(W)), "alloc output keys");
        CK(ctx->ensure(ctx->ocnt, out_cap * 4), "alloc output counts");
        const size_t p2_bytes = phase2_scratch_bytes(in);
        CK(ctx->ensure(ctx->scratch, p2_bytes), "alloc phase-2 scratch");
        P2Output po{};
        po.keys = ctx->okeys.p;
        po.counts = ctx->ocnt.as<uint32_t>();
        po.cap = out_cap;
        CK(cudaEventRecord(ctx->ev[6], ctx->st), "event");
        const tg_status ps = phase2_run(in, ctx->scratch.p, p2_bytes, po, fallback_table, ctx->st, ctx->ev[7],
                                        &launches, msg, P2Overlap());
        if (ps != TG_OK) return ctx->fail(ps, msg);
        CK(cudaEventRecord(ctx->ev[8], ctx->st), "event");
        CK(cudaEventSynchronize(ctx->ev[8]), "sync");
        cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]); T.phase2_keys_ms += ms;
        cudaEventElapsedTime(&ms, ctx->ev[7], ctx->ev[8]); T.phase2_count_ms += ms;
        const uint64_t n_p = po.n_out;
        const double c0 = now_ms();
        if (j->sink_keys || j->sink_counts) {
            const uint64_t m = acc < j->sink_cap ? std::min(n_p, j->sink_cap - acc) : 0;
            if (m && j->sink_keys)
                CK(link_copy(j->sink_keys + acc * W, po.keys, m * key_bytes(W), cudaMemcpyDeviceToHost, ctx->st,
                             ctx->n_sm), "d2h");
            if (m && j->sink_counts)
                CK(link_copy(j->sink_counts + acc, po.counts, m * 4, cudaMemcpyDeviceToHost, ctx->st, ctx->n_sm), "d2h");
            CK(cudaStreamSynchronize(ctx->st), "d2h");
        } else if (n_p) {
            j->host_keys.resize((acc + n_p) * W);
            j->host_counts.resize(acc + n_p);
            s = d2h_pageable(ctx, j->host_keys.data() + acc * W, po.keys, n_p * key_bytes(W));
            if (s == TG_OK) s = d2h_pageable(ctx, j->host_counts.data() + acc, po.counts, n_p * 4);
            if (s != TG_OK) return s;
        }
        T.d2h_ms += now_ms() - c0;
        acc += n_p;
        T.distinct += po.distinct;
        T.fallback_groups += po.fallback_groups;
        T.groups += po.groups;
        T.heavy_groups += (uint32_t)po.heavy_groups;
    }
    T.phase2_ms = now_ms() - t0;
    T.phase2_passes = passes.size();
    j->n_out = acc;
    T.bases = S.bases;
    T.runs = S.runs;
    T.kmers = S.kmers;
    T.superkmers = S.records;
    T.out = acc;
    T.gpu_parts = nb;
    T.record_bytes = S.spilled_bytes;
    T.gpu_launches = (uint64_t)(launches + j->lex_launches);
    return TG_OK;
}

tg_status tg_job_stats(const tg_job* j, tg_stats* out) {
    if (!j || !out) return TG_ERR_ARG;
    *out = j->st;
    return TG_OK;
}

uint64_t tg_job_result_size(const tg_job* j) { return j ? j->n_out : 0; }
int tg_job_key_words(const tg_job* j) { return j ? j->W : 0; }

tg_status tg_job_result_copy(tg_job* j, uint64_t* keys, uint32_t* counts, uint64_t first, uint64_t n) {
    if (!j) return TG_ERR_ARG;
    tg_ctx* ctx = j->ctx;
    if (!j->ran) return ctx->fail(TG_ERR_STATE, "result before run");
    if (first + n > j->n_out) return ctx->fail(TG_ERR_ARG, "result range out of bounds");
    if (!n) return TG_OK;
    if (j->spilled) {  // phase 2 ran in passes: the pairs are in host memory
        if (keys) parallel_copy(keys, j->host_keys.data() + first * j->W, n * 8 * (size_t)j->W, ctx->host_threads, 16u << 20);
        if (counts) parallel_copy(counts, j->host_counts.data() + first, n * 4, ctx->host_threads, 16u << 20);
        return TG_OK;
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const double t0 = now_ms();
    // jobs of several samples: the sample-major copy (each sample's pairs one range)
    const bool multi = j->sample_start.size() > 1;
    const uint8_t* kd = (multi ? ctx->okeys2 : ctx->okeys).as<uint8_t>();
    const uint32_t* cd = (multi ? ctx->ocnt2 : ctx->ocnt).as<uint32_t>();
    if (keys)
        CK(link_copy(keys, kd + first * key_bytes(j->W), n * key_bytes(j->W), cudaMemcpyDeviceToHost, ctx->st,
                     ctx->n_sm), "d2h keys");
    if (counts)
        CK(link_copy(counts, cd + first, n * 4, cudaMemcpyDeviceToHost, ctx->st, ctx->n_sm), "d2h counts");
    CK(cudaStreamSynchronize(ctx->st), "d2h");
    j->st.d2h_ms += now_ms() - t0;
    return TG_OK;
}

static tg_status tg_job_result_digest_impl(tg_job* j, uint64_t first, uint64_t n, tg_digest* out) {
    if (!j || !out) return TG_ERR_ARG;
    tg_ctx* ctx = j->ctx;
    if (!j->ran) return ctx->fail(TG_ERR_STATE, "result before run");
    if (first > j->n_out || n > j->n_out - first) return ctx->fail(TG_ERR_ARG, "result range out of bounds");
    *out = tg_digest{};
    const int W = j->W, nw = (j->o.k + 31) / 32;
    if (j->spilled) {  // the pairs are in host memory: the same terms on host threads
        const unsigned nt = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ctx->host_threads, n >> 20));
        std::vector<tg_digest> part(nt);
        auto body = [&](unsigned t) {
            const uint64_t a = first + n * t / nt, b = first + n * (t + 1) / nt;
            tg_digest d{};
            for (uint64_t i = a; i < b; ++i) {
                const uint64_t* w = j->host_keys.data() + i * W;
                uint64_t ta, tb;
                digest_terms(w[0], W > 1 ? w[1] : 0, nw, j->host_counts[i], ta, tb);
                d.h1 += ta;
                d.h2 += tb;
                d.count_sum += j->host_counts[i];
                ++d.pairs;
            }
            part[t] = d;
        };
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nt; ++t) {
            try {
                th.emplace_back(body, t);
            } catch (...) {
                body(t);
            }
        }
        body(0);
        for (auto& t : th) t.join();
        for (const tg_digest& d : part) {
            out->pairs += d.pairs;
            out->count_sum += d.count_sum;
            out->h1 += d.h1;
            out->h2 += d.h2;
        }
        return TG_OK;
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const bool multi = j->sample_start.size() > 1;
    const uint64_t* kd = (multi ? ctx->okeys2 : ctx->okeys).as<uint64_t>();
    const uint32_t* cd = (multi ? ctx->ocnt2 : ctx->ocnt).as<uint32_t>();
    unsigned long long* dd = reinterpret_cast<unsigned long long*>(ctx->misc.as<uint8_t>() + MISC_DIGEST);
    int launches = 0;
    CK(launch_digest(j->o.k, n ? kd + first * W : kd, n ? cd + first : cd, n, dd, ctx->n_sm, ctx->st, &launches),
       "k_digest");
    unsigned long long h[4];
    CK(cudaMemcpyAsync(h, dd, sizeof h, cudaMemcpyDeviceToHost, ctx->st), "d2h digest");
    CK(cudaStreamSynchronize(ctx->st), "digest");
    out->pairs = h[0];
    out->count_sum = h[1];
    out->h1 = h[2];
    out->h2 = h[3];
    return TG_OK;
}

tg_status tg_job_result_digest(tg_job* j, uint64_t first, uint64_t n, tg_digest* out) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_result_digest_impl(j, first, n, out); });
}

tg_status tg_job_sample_offsets(tg_job* j, uint64_t* offsets) {
    if (!j || !offsets) return TG_ERR_ARG;
    tg_ctx* ctx = j->ctx;
    if (!j->ran) return ctx->fail(TG_ERR_STATE, "result before run");
    const size_t ns = j->sample_start.size();
    if (ns <= 1) {
        offsets[0] = 0;
        offsets[1] = j->n_out;
        return TG_OK;
    }
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaMemcpyAsync(offsets, ctx->osoff.p, 8 * (ns + 1), cudaMemcpyDeviceToHost, ctx->st), "d2h");
    CK(cudaStreamSynchronize(ctx->st), "d2h");
    return TG_OK;
}

// Output formatting on the device in batches of DRAIN_PAIRS pairs: a batch is
// formatted into ctx->fbuf, its byte count read through mapped memory, its
// bytes copied into one of two pinned host buffers, and the previous batch is
// handed to the sink while this one copies.
constexpr uint64_t DRAIN_PAIRS = 1ull << 20;

static tg_status tg_job_drain_impl(tg_job* j, tg_format fmt, tg_sink_fn sink, void* user) {
    if (!j || !sink || (int)fmt < 0 || (int)fmt > 2) return TG_ERR_ARG;
    const TraceRange tr("tuna.drain");
    tg_ctx* ctx = j->ctx;
    if (!j->ran) return ctx->fail(TG_ERR_STATE, "drain before run");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    const uint64_t n = j->n_out;
    if (n == 0) return TG_OK;
    const int k = j->o.k, W = j->W;
    const bool multi = j->sample_start.size() > 1;
    const uint64_t* keys = (multi ? ctx->okeys2 : ctx->okeys).as<uint64_t>();
    const uint32_t* counts = (multi ? ctx->ocnt2 : ctx->ocnt).as<uint32_t>();
    const uint64_t B = std::min<uint64_t>(n, DRAIN_PAIRS);
    const size_t cap = (size_t)fmt_max_bytes((int)fmt, k, B) + 64;
    CK(ctx->ensure(ctx->fbuf, cap), "alloc format buffer");
    CK(ctx->ensure(ctx->fscr, fmt_scratch_bytes(B)), "alloc format scratch");
    if (ctx->fhost_cap < cap) {
        for (uint8_t*& h : ctx->fhost) {
            tgh::pinned_free(h);
            h = nullptr;
        }
        ctx->fhost_cap = 0;
        for (uint8_t*& h : ctx->fhost) {
            std::string why;
            h = static_cast<uint8_t*>(tgh::pinned_alloc(cap, &why));
            if (!h) return ctx->fail(TG_ERR_OOM, "pinned drain buffer: " + why);
        }
        ctx->fhost_cap = cap;
    }
    const double t0 = now_ms();
    unsigned long long* d_total = ctx->wave_out_dev + (OVERLAP_WORDS - 1);
    const volatile unsigned long long* h_total = ctx->wave_out + (OVERLAP_WORDS - 1);
    int launches = 0;
    uint64_t prev_bytes = 0, prev_pairs = 0;
    int prev = -1;
    tg_status s = TG_OK;
    const uint64_t nb = (n + B - 1) / B;
    if (j->spilled) {  // pairs in host memory: each batch is copied back to the device first
        CK(ctx->ensure(ctx->okeys, B * key_bytes(W)), "alloc");
        CK(ctx->ensure(ctx->ocnt, B * 4), "alloc");
        keys = ctx->okeys.as<uint64_t>();
        counts = ctx->ocnt.as<uint32_t>();
    }
    for (uint64_t b = 0; b < nb && s == TG_OK; ++b) {
        const uint64_t first = b * B, m = std::min(B, n - first);
        const uint64_t off = j->spilled ? 0 : first;
        if (j->spilled) {
            CK(cudaMemcpyAsync(ctx->okeys.p, j->host_keys.data() + first * W, m * key_bytes(W),
                               cudaMemcpyHostToDevice, ctx->st), "h2d");
            CK(cudaMemcpyAsync(ctx->ocnt.p, j->host_counts.data() + first, m * 4, cudaMemcpyHostToDevice, ctx->st),
               "h2d");
        }
        // the copy of batch b - 1 out of fbuf is ahead of this on the stream
        CK(launch_format((int)fmt, k, keys + off * W, counts + off, m, ctx->fbuf.as<uint8_t>(), ctx->fscr.p,
                         ctx->n_sm, ctx->st, d_total, &launches),
           "format");
        CK(cudaStreamSynchronize(ctx->st), "format");
        const uint64_t bytes = fmt == TG_FMT_TSV ? (uint64_t)*h_total : fmt_max_bytes((int)fmt, k, m);
        const int cur = (int)(b & 1);
        CK(link_copy(ctx->fhost[cur], ctx->fbuf.p, bytes, cudaMemcpyDeviceToHost, ctx->st, ctx->n_sm), "d2h");
        if (prev >= 0 && sink(ctx->fhost[prev], prev_bytes, prev_pairs, user) != 0)
            s = ctx->fail(TG_ERR_IO, "output sink stopped");
        prev = cur;
        prev_bytes = bytes;
        prev_pairs = m;
    }
    CK(cudaStreamSynchronize(ctx->st), "d2h");
    if (s == TG_OK && prev >= 0 && sink(ctx->fhost[prev], prev_bytes, prev_pairs, user) != 0)
        s = ctx->fail(TG_ERR_IO, "output sink stopped");
    j->st.d2h_ms += now_ms() - t0;
    j->st.gpu_launches += (uint64_t)launches;
    return s;
}

tg_status tg_job_drain(tg_job* j, tg_format fmt, tg_sink_fn sink, void* user) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_drain_impl(j, fmt, sink, user); });
}

struct FileSink {
    FILE* f;
};
static int file_sink(const void* data, size_t bytes, uint64_t, void* u) {
    FileSink* fs = static_cast<FileSink*>(u);
    return fwrite(data, 1, bytes, fs->f) == bytes ? 0 : 1;
}

static tg_status tg_job_write_impl(tg_job* j, tg_format fmt, const char* path) {
    if (!j || !path) return TG_ERR_ARG;
    FILE* f = fopen(path, "wb");
    if (!f) return j->ctx->fail(TG_ERR_IO, std::string("cannot open output file: ") + path);
    FileSink fs{f};
    tg_status s = TG_OK;
    if (fmt == TG_FMT_KFF) {
        const std::string h = tgh::kff_header(j->o.k, j->n_out);
        if (fwrite(h.data(), 1, h.size(), f) != h.size()) s = TG_ERR_IO;
    }
    if (s == TG_OK) s = tg_job_drain(j, fmt, file_sink, &fs);
    if (s == TG_OK && fmt == TG_FMT_KFF) {
        const std::string t = tgh::kff_footer();
        if (fwrite(t.data(), 1, t.size(), f) != t.size()) s = TG_ERR_IO;
    }
    if (fclose(f) != 0 && s == TG_OK) s = TG_ERR_IO;
    if (s == TG_ERR_IO) j->ctx->fail(s, std::string("failed while writing output file: ") + path);
    return s;
}

tg_status tg_job_write(tg_job* j, tg_format fmt, const char* path) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_write_impl(j, fmt, path); });
}

static tg_status tg_job_export_partitions_impl(tg_job* j, tg_part_sink_fn sink, void* user) {
    if (!j || !sink) return TG_ERR_ARG;
    const TraceRange tr("tuna.export_partitions");
    tg_ctx* ctx = j->ctx;
    if (!j->ran) return ctx->fail(TG_ERR_STATE, "export before run");
    if (j->sample_start.size() > 1) return ctx->fail(TG_ERR_UNSUPPORTED, "partition export of a job of several samples");
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    int launches = 0;
    // packed bases stay valid until the next run on this context
    tg_status s = run_cut(j, true, 0, &launches);
    if (s != TG_OK) return s;
    const uint32_t C = j->n_cta;
    std::vector<uint32_t> nd(C);
    CK(cudaMemcpy(nd.data(), ctx->misc.as<uint8_t>() + MISC_NDESC, (size_t)C * 4, cudaMemcpyDeviceToHost), "d2h");
    std::vector<uint32_t> pk(j->packed_words);
    CK(cudaMemcpy(pk.data(), ctx->packed.p, pk.size() * 4, cudaMemcpyDeviceToHost), "d2h packed");
    const uint32_t np = j->o.n_parts;
    std::vector<std::vector<uint8_t>> parts(np);
    std::vector<uint64_t> xd;
    const int k = j->o.k;
    const bool u16hdr = (2 * k - j->o.m) > 255;
    for (uint32_t c = 0; c < C; ++c) {
        xd.resize((size_t)nd[c] * 3);
        if (!nd[c]) continue;
        CK(cudaMemcpy(xd.data(), ctx->xdesc.as<uint64_t>() + (size_t)c * j->desc_cap * 3, xd.size() * 8,
                      cudaMemcpyDeviceToHost), "d2h");
        for (uint32_t i = 0; i < nd[c]; ++i) {
            const uint64_t st = xd[3 * i], mh = xd[3 * i + 1], x = xd[3 * i + 2];
            const uint32_t nk = (uint32_t)(x & 0xFFFFFFFFu), mp = (uint32_t)(x >> 32);
            const uint32_t len = nk + k - 1;
            std::vector<uint8_t>& out = parts[mh & (np - 1)];
            if (u16hdr) {
                const uint16_t l16 = (uint16_t)len, p16 = (uint16_t)mp;
                out.insert(out.end(), reinterpret_cast<const uint8_t*>(&l16), reinterpret_cast<const uint8_t*>(&l16) + 2);
                out.insert(out.end(), reinterpret_cast<const uint8_t*>(&p16), reinterpret_cast<const uint8_t*>(&p16) + 2);
            } else {
                out.push_back((uint8_t)len);
                out.push_back((uint8_t)mp);
            }
            const size_t o = out.size();
            out.resize(o + (len + 3) / 4, 0);
            for (uint32_t b = 0; b < len; ++b) {
                const uint64_t a = st + b + TG_PAD;
                const uint32_t code = (pk[a >> 4] >> (30 - 2 * (a & 15))) & 3u;
                out[o + (b >> 2)] |= (uint8_t)(code << (6 - 2 * (b & 3)));
            }
        }
    }
    for (uint32_t p = 0; p < np; ++p)
        if (sink(p, parts[p].data(), parts[p].size(), user) != 0) return ctx->fail(TG_ERR_IO, "partition sink stopped");
    return TG_OK;
}

tg_status tg_job_export_partitions(tg_job* j, tg_part_sink_fn sink, void* user) {
    return guarded(j ? j->ctx : nullptr, [&] { return tg_job_export_partitions_impl(j, sink, user); });
}

tg_status tg_job_end(tg_job* j) {
    if (!j) return TG_ERR_ARG;
    if (j->ctx->active == j) j->ctx->active = nullptr;
    delete j;
    return TG_OK;
}

// One job of a one-call entry point over samples [a, b) (all of tg_count_seq /
// tg_count_fastx; a run of the samples of tg_count_batch*): feed, run, results
// to keys/counts from pair `base` on (at most `cap` pairs in all), the samples'
// offsets to sample_off[a..b] (absolute). One sample: the counting pass in waves
// whose pairs are copied to the caller's buffers (on the copy stream) while the
// next waves count, the copies waited for. Several samples: the pairs are
// reordered sample-major at the end and copied then; with `pipelined` that copy
// is left running on the copy stream (ctx->ev_copied), and the next job's
// sample-major scatter waits for it, so the copy overlaps the next job's
// phases 1 and 2.
static tg_status count_run(tg_ctx* ctx, const tg_job_opts* opts, uint32_t a, uint32_t b, const uint8_t* const* seqs,
                           const size_t* lens, uint64_t* keys, uint32_t* counts, uint64_t* sample_off, uint64_t base,
                           uint64_t cap, bool fastx, bool pipelined, uint64_t& n_run, tg_stats& st_run) {
    n_run = 0;
    tg_job* j = nullptr;
    tg_status s = tg_job_begin(ctx, opts, &j);
    if (s != TG_OK) return s;
    const JobEnd end_job{j};
    const uint32_t n = b - a;
    const uint64_t room = cap > base ? cap - base : 0;
    const int W = j->W;
    uint64_t* kdst = keys ? keys + base * W : nullptr;
    uint32_t* cdst = counts ? counts + base : nullptr;
    // one buffer, separators everywhere, then every sample copied to its place
    uint64_t total = 0;
    for (uint32_t i = a; i < b; ++i) {
        if (!seqs[i] && lens[i]) s = TG_ERR_ARG;
        total += lens[i] + 1;
    }
    if (s == TG_OK && fastx) {
        // each sample's FASTA/FASTQ bytes lexed on the device into its own sample
        // (an empty sample stays empty)
        for (uint32_t i = a; i < b && s == TG_OK; ++i) {
            if (i > a) s = tg_job_next_sample(j);
            if (s == TG_OK && lens[i]) s = lex_append_host(j, seqs[i], lens[i]);
        }
    } else if (s == TG_OK && total) {
        const double t0 = now_ms();
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e == cudaSuccess) e = ctx->ensure(ctx->seq, total + 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->seq.p, '\n', total, ctx->st);
        uint64_t off = 0;
        for (uint32_t i = a; i < b && e == cudaSuccess; ++i) {
            if (i > a) j->sample_start.push_back(off);
            if (lens[i])
                e = link_copy(ctx->seq.as<uint8_t>() + off, seqs[i], lens[i], cudaMemcpyHostToDevice, ctx->st, ctx->n_sm);
            off += lens[i] + 1;
            j->st.input_bytes += lens[i];
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e != cudaSuccess) s = ctx->cuda_fail(e, "copy input");
        j->n = total;
        j->used_ctx_seq = true;
        j->st.h2d_ms += now_ms() - t0;
    }
    P2Overlap ov;
    ov.waves = 8;
    ov.wave_out = ctx->wave_out;
    ov.wave_out_dev = ctx->wave_out_dev;
    ov.wave_ev = ctx->wave_ev;
    double d2h_issue_ms = 0;
    const bool multi = n > 1;
    ov.on_range = [&](uint64_t lo, uint64_t hi) -> tg_status {
        const uint64_t h = std::min<uint64_t>(hi, room);
        if (h <= lo) return TG_OK;
        const double t0 = now_ms();
        if (kdst)
            CK(link_copy(kdst + lo * W, ctx->okeys.as<uint8_t>() + lo * key_bytes(W), (h - lo) * key_bytes(W),
                         cudaMemcpyDeviceToHost, ctx->st_copy, ctx->n_sm), "d2h keys");
        if (cdst)
            CK(link_copy(cdst + lo, ctx->ocnt.as<uint32_t>() + lo, (h - lo) * 4, cudaMemcpyDeviceToHost,
                         ctx->st_copy, ctx->n_sm), "d2h counts");
        d2h_issue_ms += now_ms() - t0;
        return TG_OK;
    };
    j->overlap = multi ? nullptr : &ov;
    j->reorder_after = multi && ctx->copy_pending ? ctx->ev_copied : nullptr;
    // a run in passes (memory budget) copies each pass's pairs here itself
    j->sink_keys = kdst;
    j->sink_counts = cdst;
    j->sink_cap = room;
    if (s == TG_OK) s = tg_job_run(j);
    if (s == TG_OK && multi) {
        const uint64_t h = std::min<uint64_t>(j->n_out, room);
        const double t0 = now_ms();
        if (h && (kdst || cdst)) {
            if (pipelined && !j->spilled) {
                // the run left the sample-major pairs in okeys2/ocnt2 and its stream idle;
                // pending from the first copy on, so that any return waits for it
                ctx->copy_pending = true;
                if (kdst)
                    CK(link_copy(kdst, ctx->okeys2.as<uint8_t>(), h * key_bytes(W), cudaMemcpyDeviceToHost,
                                 ctx->st_copy, ctx->n_sm), "d2h keys");
                if (cdst)
                    CK(link_copy(cdst, ctx->ocnt2.as<uint32_t>(), h * 4, cudaMemcpyDeviceToHost, ctx->st_copy,
                                 ctx->n_sm), "d2h counts");
                CK(cudaEventRecord(ctx->ev_copied, ctx->st_copy), "event");
            } else {
                s = tg_job_result_copy(j, kdst, cdst, 0, h);
            }
        }
        if (s == TG_OK && sample_off) {
            std::vector<uint64_t> off(n + 1);
            s = tg_job_sample_offsets(j, off.data());
            for (uint32_t i = 0; i <= n && s == TG_OK; ++i) sample_off[a + i] = base + off[i];
        }
        d2h_issue_ms += now_ms() - t0;
    }
    if (!pipelined || !multi) {
        const double t_wait = now_ms();
        const cudaError_t ce = cudaStreamSynchronize(ctx->st_copy);
        j->st.d2h_ms += now_ms() - t_wait;
        if (s == TG_OK && ce != cudaSuccess) s = ctx->cuda_fail(ce, "d2h");
        ctx->copy_pending = false;
    }
    j->st.d2h_ms += d2h_issue_ms;
    if (s == TG_OK) {
        n_run = j->n_out;
        if (sample_off && !multi) { sample_off[a] = base; sample_off[b] = base + j->n_out; }
    }
    st_run = j->st;
    return s;
}

// Sums the counters and times of one run of a batch into the batch's stats.
static void add_run_stats(tg_stats& t, const tg_stats& r) {
    t.input_bytes += r.input_bytes;
    t.bases += r.bases;
    t.runs += r.runs;
    t.kmers += r.kmers;
    t.superkmers += r.superkmers;
    t.distinct += r.distinct;
    t.out += r.out;
    t.gpu_parts = r.gpu_parts;
    t.heavy_groups += r.heavy_groups;
    t.fallback_groups += r.fallback_groups;
    t.h2d_ms += r.h2d_ms;
    t.pack_ms += r.pack_ms;
    t.phase1_ms += r.phase1_ms;
    t.phase2_ms += r.phase2_ms;
    t.d2h_ms += r.d2h_ms;
    t.phase1_cut_ms += r.phase1_cut_ms;
    t.phase1_scatter_ms += r.phase1_scatter_ms;
    t.record_bytes += r.record_bytes;
    t.gpu_launches += r.gpu_launches;
    t.phase2_count_ms += r.phase2_count_ms;
    t.phase2_keys_ms += r.phase2_keys_ms;
    t.groups += r.groups;
    t.lex_ms += r.lex_ms;
    t.fastx_bytes += r.fastx_bytes;
    t.host_parsed_bytes += r.host_parsed_bytes;
    t.phase2_passes = std::max(t.phase2_passes, r.phase2_passes);
    t.group_load_pct = r.group_load_pct;
    t.autotune_trials += r.autotune_trials;
}

// A batch (several samples) larger than the device budget runs as
// consecutive runs of samples of at most budget / BATCH_BYTES_PER_BASE input
// bytes (a job of several samples is not counted in passes, so each run must
// fit; a sample is never split), each run's result copy left running while the
// next run counts. Cutting batches that fit into runs as well, only to overlap
// the copies, was measured slower: the copy kernels cannot sit beside the cut
// and key kernels on an SM (registers), so little overlapped, and smaller jobs
// cost more (2,000 samples, 1.23 Gbp: 40 -> 73 ms in four runs).
constexpr uint64_t BATCH_BYTES_PER_BASE = 40;  // keys, pairs and their sample-major copy, records, stream

// The one-call entry points.
static tg_status count_host(tg_ctx* ctx, const tg_job_opts* opts, uint32_t n_samples, const uint8_t* const* seqs,
                            const size_t* lens, uint64_t* keys, uint32_t* counts, uint64_t* sample_off, uint64_t cap,
                            uint64_t* n_out, tg_stats* stats, bool fastx = false) {
    if (!ctx || !opts || !n_out || (n_samples && (!seqs || !lens))) return TG_ERR_ARG;
    *n_out = 0;
    if (n_samples > TG_MAX_SAMPLES) return ctx->fail(TG_ERR_ARG, "too many samples in one job");
    uint64_t total = 0;
    for (uint32_t i = 0; i < n_samples; ++i) total += lens[i];
    // runs of samples [cut[r], cut[r + 1])
    std::vector<uint32_t> cut{0};  // tg_count_batch* take at least one sample, the others exactly one
    uint64_t target = ~0ull;
    if (n_samples > 1) {
        CK(cudaSetDevice(ctx->device), "cudaSetDevice");
        uint64_t budget = 0;
        const tg_status bs = phase2_budget(ctx, &budget);
        if (bs != TG_OK) return bs;
        target = std::max<uint64_t>(1, budget / BATCH_BYTES_PER_BASE);
    }
    if (total > target) {
        uint64_t acc = 0;
        for (uint32_t i = 0; i < n_samples; ++i) {
            if (acc && acc + lens[i] > target) {
                cut.push_back(i);
                acc = 0;
            }
            acc += lens[i];
        }
    }
    cut.push_back(n_samples);
    const bool pipelined = cut.size() > 2;
    tg_stats all{};
    uint64_t done = 0;
    tg_status s = TG_OK;
    for (size_t r = 0; r + 1 < cut.size() && s == TG_OK; ++r) {
        uint64_t nr = 0;
        tg_stats sr{};
        s = count_run(ctx, opts, cut[r], cut[r + 1], seqs, lens, keys, counts, sample_off, done, cap, fastx,
                      pipelined, nr, sr);
        if (r == 0) all = sr;
        else add_run_stats(all, sr);
        done += nr;
    }
    if (ctx->copy_pending) {
        const double t_wait = now_ms();
        const cudaError_t ce = cudaStreamSynchronize(ctx->st_copy);
        all.d2h_ms += now_ms() - t_wait;
        ctx->copy_pending = false;
        if (s == TG_OK && ce != cudaSuccess) s = ctx->cuda_fail(ce, "d2h");
    }
    if (s == TG_OK) {
        *n_out = done;
        if (done > cap) s = ctx->fail(TG_ERR_ARG, "result buffer too small");
    }
    if (stats) *stats = all;
    return s;
}

tg_status tg_count_seq(tg_ctx* ctx, const tg_job_opts* opts, const uint8_t* seq, size_t len, uint64_t* keys,
                       uint32_t* counts, uint64_t cap, uint64_t* n_out, tg_stats* stats) {
    if (!seq && len) return TG_ERR_ARG;
    return guarded(ctx, [&] { return count_host(ctx, opts, 1, &seq, &len, keys, counts, nullptr, cap, n_out, stats); });
}

tg_status tg_count_fastx(tg_ctx* ctx, const tg_job_opts* opts, const uint8_t* data, size_t len, uint64_t* keys,
                         uint32_t* counts, uint64_t cap, uint64_t* n_out, tg_stats* stats) {
    if (!data && len) return TG_ERR_ARG;
    return guarded(ctx, [&] { return count_host(ctx, opts, 1, &data, &len, keys, counts, nullptr, cap, n_out, stats, true); });
}

tg_status tg_count_batch_fastx(tg_ctx* ctx, const tg_job_opts* opts, uint32_t n_samples,
                               const uint8_t* const* datas, const size_t* lens, uint64_t* keys, uint32_t* counts,
                               uint64_t* sample_offsets, uint64_t cap, uint64_t* n_out, tg_stats* stats) {
    if (n_samples == 0) return TG_ERR_ARG;
    return guarded(ctx, [&] { return count_host(ctx, opts, n_samples, datas, lens, keys, counts, sample_offsets, cap, n_out, stats, true); });
}

tg_status tg_count_batch(tg_ctx* ctx, const tg_job_opts* opts, uint32_t n_samples, const uint8_t* const* seqs,
                         const size_t* lens, uint64_t* keys, uint32_t* counts, uint64_t* sample_offsets, uint64_t cap,
                         uint64_t* n_out, tg_stats* stats) {
    if (n_samples == 0) return TG_ERR_ARG;
    return guarded(ctx, [&] { return count_host(ctx, opts, n_samples, seqs, lens, keys, counts, sample_offsets, cap, n_out, stats); });
}

}  // extern "C"
