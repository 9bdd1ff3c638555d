// tg_noalloc.cu — counting without any device allocation, for callers that
// must not allocate.
//
// Who needs it: code that runs where a cudaMalloc/cudaFree is not allowed or
// not wanted at call time — an inference-server or plugin `enqueue` that is
// handed its buffers and a stream and may not allocate, a process whose device
// memory is owned by another allocator (a framework's caching allocator, a
// pre-reserved pool), or a latency-critical loop where an allocation would
// synchronise the device. tg_count_seq_device_noalloc takes the input and the
// output buffers from the caller and keeps every intermediate array (packed
// bases, superkmer descriptors, the bin histogram and key offsets,
// k-mer keys, group lists, fallback table) in one file-scope device array of
// TG_NOALLOC_SCRATCH_BYTES that stays reserved until the process exits. The CUDA
// runtime loads this file's module, and so reserves the array, on a device the
// first time the array's address is looked up there, which is the first call on
// that device (or at library load with CUDA_MODULE_LOADING=EAGER): that first
// call does allocate. A call with len == 0 does only this, so a caller makes it
// once per device before its own allocator takes the device's memory.
//
// It runs the same kernels as tg_job_run on the same parameters, so its output
// is the same set of (k-mer, count) pairs: the counting of run_callback<k,m>
// (src/pipeline.hpp:273-330 of the reference) over a sequence stream. Inputs longer than
// TG_NOALLOC_MAX_LEN bytes are rejected; so is an input whose intermediate
// arrays would not fit in the scratch array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "tg_internal.cuh"
#include "tg_launch.h"
#include "tuna_gpu.h"

using namespace tg;

// All scratch of the entry point. In host code this name is only a handle for
// cudaGetSymbolAddress: its device address is looked up per device at first use.
static __device__ __align__(256) uint8_t tg_noalloc_scratch[TG_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
constexpr int MAX_DEV = 64;
uint8_t* g_scratch_addr[MAX_DEV] = {};

void set_err(char* buf, size_t len, const std::string& msg) {
    if (buf && len) {
        const size_t n = std::min(len - 1, msg.size());
        memcpy(buf, msg.data(), n);
        buf[n] = 0;
    }
}

// Device address of the scratch array on the current device (looked up once per
// device, with that device current).
cudaError_t scratch_address(int dev, uint8_t** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, tg_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<uint8_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

// Bump allocator over the scratch array (256-byte aligned pieces).
struct Carve {
    uint8_t* base;
    size_t off = 0, cap;
    bool ok = true;
    template <typename T>
    T* take(size_t count) {
        const size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        if (!ok || off + bytes > cap) { ok = false; return nullptr; }
        T* p = reinterpret_cast<T*>(base + off);
        off += bytes;
        return p;
    }
};

}  // namespace

static tg_status count_noalloc(const tg_job_opts* opts, const uint8_t* d_seq, size_t len, uint64_t* d_keys,
                               uint32_t* d_counts, uint64_t cap, uint64_t* n_out, void* stream, char* errbuf,
                               size_t errlen) {
    if (!opts || !n_out || (!d_seq && len)) { set_err(errbuf, errlen, "null argument"); return TG_ERR_ARG; }
    *n_out = 0;
    const tg_job_opts& o = *opts;
    if (o.k < 2 || o.k > 63 || o.m < 1 || o.m > 32 || o.m >= o.k) {
        set_err(errbuf, errlen, "k must be in [2, 63] and m in [1, min(k-1, 32)]");
        return o.k > 63 ? TG_ERR_UNSUPPORTED : TG_ERR_ARG;
    }
    // the same rule as tg_job_begin: 0 (auto) or a power of two up to P1_MAX
    if (o.gpu_parts && ((o.gpu_parts & (o.gpu_parts - 1)) || o.gpu_parts > (uint32_t)P1_MAX)) {
        set_err(errbuf, errlen, "gpu_parts must be 0 or a power of two <= " + std::to_string(P1_MAX));
        return TG_ERR_ARG;
    }
    if (len > TG_NOALLOC_MAX_LEN) {
        set_err(errbuf, errlen, "input of " + std::to_string(len) + " bytes exceeds the no-allocation limit of " +
                                    std::to_string(TG_NOALLOC_MAX_LEN) + " bytes");
        return TG_ERR_ARG;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEV) { set_err(errbuf, errlen, "no current CUDA device"); return TG_ERR_CUDA; }
    uint8_t* base = nullptr;
    e = scratch_address(dev, &base);
    if (e != cudaSuccess) {
        set_err(errbuf, errlen, std::string("cudaGetSymbolAddress (reserving the scratch array on this device): ") +
                                    cudaGetErrorString(e));
        return TG_ERR_CUDA;
    }
    // an empty input: nothing to count. A call with len == 0 is the warm-up that
    // reserves the scratch array on the current device (see tuna_gpu.h).
    if (len == 0) return TG_OK;
    int n_sm = 0;
    e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n_sm <= 0) {
        set_err(errbuf, errlen, std::string("multiprocessor count: ") + cudaGetErrorString(e));
        return TG_ERR_CUDA;
    }
#define NA_CK(call, what)                                                                          \
    do {                                                                                           \
        const cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) { set_err(errbuf, errlen, std::string(what) + ": " + cudaGetErrorString(e_)); return TG_ERR_CUDA; } \
    } while (0)
    const int k = o.k, m = o.m, w = k - m, W = k <= 31 ? 1 : 2;
    const uint32_t hdr_max = (2u * k - m <= 255u) ? 255u : 65535u;
    const uint32_t L = hdr_max + 1 - k;
    const uint64_t n = len;
    Carve cv{base, 0, (size_t)TG_NOALLOC_SCRATCH_BYTES};
    // ---- fixed pieces
    HashTables* tables = cv.take<HashTables>(1);
    unsigned long long* misc = cv.take<unsigned long long>(32);  // counters, see below
    const uint64_t pw = packed_words_for(n);
    uint32_t* packed = cv.take<uint32_t>(pw);
    uint32_t* valid = cv.take<uint32_t>(pw / 2 + 16);
    // phase-1 layout: as tg_job_run, with room for one record per k-mer start
    uint32_t p1 = o.gpu_parts ? o.gpu_parts : std::min<uint32_t>(1024, std::max<uint32_t>(16, (uint32_t)(n / 32768)));
    uint32_t p1_bits = 0;
    while ((1u << p1_bits) < p1) ++p1_bits;
    p1 = 1u << p1_bits;
    const uint64_t tile = cut_tile(w, false);
    uint32_t C = (uint32_t)n_sm * cut_ctas_per_sm(w, k, p1, false);
    uint64_t chunk = (n + C - 1) / C;
    chunk = std::max<uint64_t>(tile, (chunk + tile - 1) / tile * tile);
    C = (uint32_t)std::max<uint64_t>(1, (n + chunk - 1) / chunk);
    const uint64_t desc_cap = chunk + 2ull * tile + L + 64;
    uint64_t* desc = cv.take<uint64_t>((size_t)C * desc_cap);
    uint32_t* n_desc = cv.take<uint32_t>(C);
    uint32_t* binhist = cv.take<uint32_t>((size_t)1 << BIN_BITS);
    // one sample: all 2^20 bins, cut into p1 segments
    const SampleBins B = layout_bins({0ull, (unsigned long long)n}, (1u << BIN_BITS) >> p1_bits);
    unsigned long long* s_start = cv.take<unsigned long long>(2);
    uint32_t* s_base = cv.take<uint32_t>(1);
    uint8_t* s_bits = cv.take<uint8_t>(1);
    if (!cv.ok) { set_err(errbuf, errlen, "input too large for the no-allocation scratch"); return TG_ERR_ARG; }
    // counters in misc (u64 indices): [0..2] k-mers/records/runs, [3] bases, [4] overflow (u32)
    uint32_t* overflow = reinterpret_cast<uint32_t*>(misc + 4);

    const HashTables T = make_hash_tables(m);
    NA_CK(cudaMemcpyAsync(tables, &T, sizeof T, cudaMemcpyHostToDevice, st), "upload tables");
    NA_CK(cudaMemsetAsync(misc, 0, 32 * 8, st), "memset");
    NA_CK(cudaMemsetAsync(binhist, 0, (size_t)4 << BIN_BITS, st), "memset");
    NA_CK(cudaMemcpyAsync(s_start, B.start.data(), 16, cudaMemcpyHostToDevice, st), "h2d");
    NA_CK(cudaMemcpyAsync(s_base, B.base.data(), 4, cudaMemcpyHostToDevice, st), "h2d");
    NA_CK(cudaMemcpyAsync(s_bits, B.bits.data(), 1, cudaMemcpyHostToDevice, st), "h2d");
    // ---- phase 1
    NA_CK(launch_pack(d_seq, n, packed, valid, pw, misc + 3, st), "k_pack");
    CutParams P{};
    P.packed = packed; P.valid = valid; P.n = n;
    P.k = k; P.m = m; P.w = w; P.L = L;
    P.p1_bits = p1_bits; P.n_cta = C; P.chunk = chunk;
    P.desc = desc; P.desc_cap = desc_cap; P.n_desc = n_desc;
    P.hist = nullptr; P.binhist = binhist; P.stats = misc; P.overflow = overflow; P.xdesc = nullptr;
    P.sample_start = s_start; P.sample_bin_base = s_base; P.sample_bin_bits = s_bits; P.n_samples = 1;
    NA_CK(launch_cut(P, tables, false, st), "k_cut");
    int launches = 0;
    std::vector<uint32_t> nd(C);
    unsigned long long cstats[3] = {0, 0, 0};
    uint32_t ovf = 0;
    NA_CK(cudaMemcpyAsync(nd.data(), n_desc, (size_t)C * 4, cudaMemcpyDeviceToHost, st), "d2h");
    NA_CK(cudaMemcpyAsync(cstats, misc, 24, cudaMemcpyDeviceToHost, st), "d2h");
    NA_CK(cudaMemcpyAsync(&ovf, overflow, 4, cudaMemcpyDeviceToHost, st), "d2h");
    NA_CK(cudaStreamSynchronize(st), "phase 1");
    if (ovf) { set_err(errbuf, errlen, "descriptor capacity exceeded"); return TG_ERR_DEVICE; }
    // ---- phase 2 in what is left
    P2Input in{};
    in.W = W; in.k = k; in.segs = B.segs.data(); in.n_segs = (uint32_t)B.segs.size(); in.n_sm = (uint32_t)n_sm;
    in.packed = packed; in.desc = desc; in.desc_cap = desc_cap; in.n_lists = C; in.n_desc = nd.data();
    in.binhist = binhist; in.n_kmers = cstats[0];
    in.ci = o.ci; in.cx = o.cx;
    const size_t p2_bytes = phase2_scratch_bytes(in);
    uint8_t* p2_scratch = cv.take<uint8_t>(p2_bytes);
    if (!cv.ok) { set_err(errbuf, errlen, "input too large for the no-allocation scratch"); return TG_ERR_ARG; }
    // a global table for a group that overflows shared memory: the space after
    // the phase-2 scratch, reused by each such group in turn
    const size_t fb_base = cv.off;
    auto fallback_table = [&](size_t bytes) -> void* {
        cv.off = fb_base;
        cv.ok = true;
        return cv.take<uint8_t>(bytes);
    };
    P2Output out{};
    out.keys = d_keys; out.counts = d_counts; out.cap = cap;
    std::string msg;
    // straight into the caller's buffers
    const tg_status ps = phase2_run(in, p2_scratch, p2_bytes, out, fallback_table, st, nullptr, &launches, msg);
    *n_out = out.n_out;
    if (ps != TG_OK) {
        if (out.n_out > cap) {
            set_err(errbuf, errlen, "output capacity too small: " + std::to_string(out.n_out) + " k-mers");
            return TG_ERR_ARG;
        }
        set_err(errbuf, errlen, msg);
        return ps;
    }
#undef NA_CK
    return TG_OK;
}

// Host-side C++ failures (the bin layout's vectors, messages) become a status:
// no exception crosses the C ABI.
extern "C" tg_status tg_count_seq_device_noalloc(const tg_job_opts* opts, const uint8_t* d_seq, size_t len,
                                                 uint64_t* d_keys, uint32_t* d_counts, uint64_t cap,
                                                 uint64_t* n_out, void* stream, char* errbuf, size_t errlen) {
    try {
        return count_noalloc(opts, d_seq, len, d_keys, d_counts, cap, n_out, stream, errbuf, errlen);
    } catch (const std::exception& x) {
        if (errbuf && errlen) snprintf(errbuf, errlen, "host: %s", x.what());
    } catch (...) {
        if (errbuf && errlen) snprintf(errbuf, errlen, "host: unknown exception");
    }
    return TG_ERR_OOM;
}
