// tg_launch.h — host-side launchers of the counting kernels (defined in
// tg_phase1.cu, tg_phase2.cu, tg_api.cu) shared by the entry points.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "tuna_gpu.h"

#include "tg_internal.cuh"

namespace tg {
size_t cut_smem_bytes(int w, int k, uint32_t p1, bool exp);
uint64_t cut_tile(int w, bool exp);                 // k-mer start positions per tile of a cut CTA
uint32_t cut_ctas_per_sm(int w, int k, uint32_t p1, bool exp);
// Packed words (a multiple of 4) for a stream of n bytes, padding included.
uint64_t packed_words_for(uint64_t n);
cudaError_t launch_pack(const uint8_t* seq, uint64_t n, uint32_t* packed, uint32_t* valid, uint64_t n_words,
                        unsigned long long* n_bases, cudaStream_t st);
cudaError_t launch_cut(const CutParams& P, const HashTables* gT, bool exp, cudaStream_t st);
cudaError_t launch_scan(const uint32_t* in, uint64_t n, unsigned long long* out, unsigned long long* sums,
                        unsigned long long* total, cudaStream_t st, int* launches);
// FASTA/FASTQ lexing on the device (tg_lex.cu). raw must be 16-byte aligned;
// out receives at most len bytes. Totals are written to device memory (*dtot,
// inside scratch) and are valid once the stream reaches them.
struct LexTotals {
    unsigned long long out;        // stream bytes written
    unsigned long long drop_from;  // FASTQ: bytes from here on were not emitted (end-of-file rule)
    uint32_t final_state;          // automaton state at the end of the file
    uint32_t irregular;            // bit 0: FASTQ with an empty header line at offset 63 mod 64 (parse
                                   // on the host); bit 1: a staging wait timed out (device error)
};
size_t lex_scratch_bytes(uint64_t len);
cudaError_t launch_lex(const uint8_t* raw, uint64_t len, bool fastq, uint8_t* out, void* scratch, int n_sm,
                       cudaStream_t st, LexTotals** dtot, int* launches);
// Output formatting on the device (tg_format.cu): n pairs to the bytes of
// format fmt (tg_format). TSV writes its byte count to d_total (device-
// writable, e.g. mapped host memory); KFF and RAW records have a fixed size,
// fmt_max_bytes, and leave d_total alone.
size_t fmt_scratch_bytes(uint64_t n_pairs);
uint64_t fmt_max_bytes(int fmt, int k, uint64_t n_pairs);
cudaError_t launch_format(int fmt, int k, const uint64_t* keys, const uint32_t* counts, uint64_t n, uint8_t* out,
                          void* scratch, int n_sm, cudaStream_t st, unsigned long long* d_total, int* launches);
// Digest of n pairs (tg_job_result_digest) into out[4] (device): pairs, count
// sum, h1, h2.
cudaError_t launch_digest(int k, const uint64_t* keys, const uint32_t* counts, uint64_t n, unsigned long long* out,
                          int n_sm, cudaStream_t st, int* launches);
// A copy between device memory and host memory (tg_link.cu): done by a kernel
// through the mapped address when the host side is page-locked memory mapped
// for the current device (and both sides are equally aligned mod 16), else by
// cudaMemcpyAsync; ordered on st like cudaMemcpyAsync.
cudaError_t link_copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st, int n_sm,
                      int* launches = nullptr);
// The device address of host memory that is page-locked and mapped for the
// current device, else null (pageable memory, device memory, bad pointers).
const void* mapped_address(const void* host);
// Spill mode (tg_spill.cu): records of the phase-1 descriptor lists to
// per-bucket staging areas (bucket = bin >> shift, at most SPILL_MAX_BUCKETS).
// launch_spill_size: totals[b] records and totals[nb + b] bytes of bucket b.
// launch_spill_write: cursors[b] / cursors[nb + b] start at bucket b's staging
// base (records / bytes); host_shift[b] = the bucket stream's length before
// this chunk minus its staging byte base; staging byte bases and stream lengths
// are multiples of 4. launch_rebase: add `add` to the start of n descriptors.
constexpr uint32_t SPILL_MAX_BUCKETS = 1024;
cudaError_t launch_spill_size(const uint64_t* desc, uint64_t desc_cap, const uint32_t* n_desc, uint32_t n_lists,
                              int k, int shift, uint32_t nb, unsigned long long* totals, cudaStream_t st);
cudaError_t launch_spill_write(const uint32_t* packed, const uint64_t* desc, uint64_t desc_cap, const uint32_t* n_desc,
                               uint32_t n_lists, int k, int shift, uint32_t nb, unsigned long long* cursors,
                               const long long* host_shift, uint64_t* out_desc, uint8_t* out_bytes, cudaStream_t st);
cudaError_t launch_rebase(uint64_t* desc, uint64_t n, uint64_t add, int n_sm, cudaStream_t st);
size_t key_bytes(int W);
uint32_t count_slots(int W);

// Phase 2 of one job, shared by the entry points: the phase-1 descriptor lists
// and the k-mer counts per bin in, distinct keys and counts (and their
// samples) out.
// Bins of one sample per segment; the host helper below lays them out.
struct SampleBins {
    std::vector<unsigned long long> start;  // [n + 1] stream position of each sample, then the end
    std::vector<uint32_t> base;             // [n] first bin
    std::vector<uint8_t> bits;              // [n] log2 bins
    std::vector<Segment> segs;
};
// Shares the 2^20 bins out among samples in proportion to their length (a
// power of two each) and cuts each sample's bins into segments of at most
// seg_bins bins.
SampleBins layout_bins(const std::vector<unsigned long long>& sample_start, uint32_t seg_bins);
struct P2Input {
    int W, k;                          // key words, k
    const Segment* segs;               // [n_segs] (host): runs of bins of one sample, cut into groups
    uint32_t n_segs;
    uint32_t n_sm;
    const uint32_t* packed;
    const uint64_t* desc;              // [n_lists][desc_cap] phase-1 descriptors
    uint64_t desc_cap;
    uint32_t n_lists;
    const uint32_t* n_desc;            // [n_lists] descriptors per list (host)
    const uint32_t* binhist;           // [2^20] k-mers per bin (device)
    uint64_t n_kmers;                  // k-mer instances in all
    uint64_t ci, cx;
    uint32_t n_samples = 1;
    // the bins counted by this run (all by default); segs must lie inside and
    // n_kmers count only their keys
    uint32_t bin_lo = 0, bin_hi = 1u << BIN_BITS;
    uint32_t group_pct = 50;  // keys per group, % of the table's slots
};
struct P2Output {
    void* keys;                        // u64 x W per distinct k-mer
    uint32_t* counts;
    uint32_t* samples = nullptr;       // sample of each pair, or null
    // jobs of several samples: the pairs again, sample-major, and the first pair
    // of each sample (n_samples + 1 entries, device)
    uint32_t n_samples = 1;
    void* keys2 = nullptr;
    uint32_t* counts2 = nullptr;
    unsigned long long* sample_off = nullptr;
    uint64_t cap;
    uint64_t n_out, distinct, groups, heavy_groups, fallback_groups;
    // the sample-major scatter waits for this event first (an earlier job's
    // copy of keys2/counts2 to the host may still be running), or null
    cudaEvent_t reorder_after = nullptr;
};
// Results handed out while phase 2 still runs: the first counting pass runs in
// `waves` launches, and after each one on_range(lo, hi) is called (on the host,
// in order) with the output range [lo, hi) that is now final in P2Output;
// the last call comes after the retry passes. wave_out: pinned host memory of
// `waves` u64; wave_ev: `waves` events. Empty on_range: one launch, no calls.
struct P2Overlap {
    uint32_t waves = 1;
    unsigned long long* wave_out = nullptr;      // host address of mapped pinned memory, OVERLAP_WORDS u64
    unsigned long long* wave_out_dev = nullptr;  // its device address
    cudaEvent_t* wave_ev = nullptr;
    std::function<tg_status(uint64_t lo, uint64_t hi)> on_range;
};
// wave_out layout: [0, 16) output totals after each wave, [16, 64) counter reads.
// Counters are read back by a one-warp kernel storing into this mapped memory,
// not by cudaMemcpyAsync: a copy-engine read would queue behind the result
// copies already issued on the copy stream.
constexpr uint32_t OVERLAP_WORDS = 64;
// Device scratch one run needs (key array included).
size_t phase2_scratch_bytes(const P2Input& in);
// Runs phase 2 on `st` and waits for it. fallback_table(bytes) returns device
// memory for a global table (or null); ev_keys (optional) is recorded once the
// keys are written.
tg_status phase2_run(const P2Input& in, void* scratch, size_t scratch_cap, P2Output& out,
                     const std::function<void*(size_t)>& fallback_table, cudaStream_t st, cudaEvent_t ev_keys,
                     int* launches, std::string& err, const P2Overlap& ov = P2Overlap());

// ntHash roll / init tables for minimizer length m (host side).
HashTables make_hash_tables(int m);

}  // namespace tg
