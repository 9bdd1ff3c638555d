// tg_spill.cu — the kernels of spill mode (tg_job_set_spill): superkmer
// records of one chunk of input moved out of the chunk's packed stream into
// per-bucket record streams, and the descriptors of uploaded buckets rebased.
//
// Reference counterpart: the disk pipeline of src/pipeline.hpp:186-263, whose
// phase 1 appends every superkmer to the file of its partition
// (SuperkmerWriter::append_kache, src/superkmer_io.hpp:154-172) and whose
// phase 2 replays one partition file at a time (SuperkmerReader,
// src/superkmer_io.hpp:196-266). Here a bucket is a run of consecutive bins
// (minimizer-hash bits, the role of the partition id); a record keeps its bases
// (2-bit, four per byte, in the byte order of the packed u32 words, so that a
// bucket stream uploaded at a 16-base boundary is a packed stream again) and a
// descriptor (start in its bucket stream, k-mers, bin).
#include <cstdint>

#include "tg_launch.h"

namespace tg {
namespace {

constexpr int SPILL_THREADS = 256;

__device__ __forceinline__ uint32_t spill_bucket(uint64_t d, int shift) { return desc_bin(d) >> shift; }

__device__ __forceinline__ uint32_t record_bytes(uint64_t d, int k) { return (desc_nk(d) + (uint32_t)k - 1 + 3) / 4; }

// Per-bucket records and bytes of all descriptor lists (one CTA per list).
__global__ void __launch_bounds__(SPILL_THREADS) k_spill_size(const uint64_t* __restrict__ desc, uint64_t desc_cap,
                                                              const uint32_t* __restrict__ n_desc, int k, int shift,
                                                              uint32_t nb, unsigned long long* __restrict__ totals) {
    __shared__ unsigned long long s_rec[SPILL_MAX_BUCKETS], s_bytes[SPILL_MAX_BUCKETS];
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) { s_rec[b] = 0; s_bytes[b] = 0; }
    __syncthreads();
    const uint64_t* d = desc + (uint64_t)blockIdx.x * desc_cap;
    const uint32_t n = n_desc[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t v = d[i];
        const uint32_t b = spill_bucket(v, shift);
        atomicAdd(&s_rec[b], 1ull);
        atomicAdd(&s_bytes[b], (unsigned long long)record_bytes(v, k));
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        if (s_rec[b]) atomicAdd(&totals[b], s_rec[b]);
        if (s_bytes[b]) atomicAdd(&totals[nb + b], s_bytes[b]);
    }
}

// Every record of the lists to its bucket's staging range: descriptor (start =
// 4 x its byte position in the bucket's whole stream) and bases. cursors[b] /
// cursors[nb + b]: the next free record / byte of bucket b in the staging
// buffers (start at the bucket's staging base); host_bytes[b]: the bucket
// stream's length before this chunk, minus its staging base.
__global__ void __launch_bounds__(SPILL_THREADS) k_spill_write(const uint32_t* __restrict__ packed,
                                                               const uint64_t* __restrict__ desc, uint64_t desc_cap,
                                                               const uint32_t* __restrict__ n_desc, int k, int shift,
                                                               uint32_t nb, unsigned long long* __restrict__ cursors,
                                                               const long long* __restrict__ host_shift,
                                                               uint64_t* __restrict__ out_desc,
                                                               uint8_t* __restrict__ out_bytes) {
    __shared__ unsigned long long s_rec[SPILL_MAX_BUCKETS], s_bytes[SPILL_MAX_BUCKETS];
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) { s_rec[b] = 0; s_bytes[b] = 0; }
    __syncthreads();
    const uint64_t* d = desc + (uint64_t)blockIdx.x * desc_cap;
    const uint32_t n = n_desc[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t v = d[i];
        const uint32_t b = spill_bucket(v, shift);
        atomicAdd(&s_rec[b], 1ull);
        atomicAdd(&s_bytes[b], (unsigned long long)record_bytes(v, k));
    }
    __syncthreads();
    // this CTA's ranges in the buckets' staging areas
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        s_rec[b] = s_rec[b] ? atomicAdd(&cursors[b], s_rec[b]) : 0;
        s_bytes[b] = s_bytes[b] ? atomicAdd(&cursors[nb + b], s_bytes[b]) : 0;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t v = d[i];
        const uint32_t b = spill_bucket(v, shift);
        const uint32_t nbytes = record_bytes(v, k);
        const unsigned long long r = atomicAdd(&s_rec[b], 1ull);
        const unsigned long long p = atomicAdd(&s_bytes[b], (unsigned long long)nbytes);  // staging byte
        const unsigned long long in_stream = (unsigned long long)((long long)p + host_shift[b]);
        out_desc[r] = desc_pack(4ull * in_stream, desc_nk(v), desc_bin(v));
        // bases [start, start + nk + k - 1), 32 per window, 4 per byte; byte j of a
        // stream sits at (j & ~3) + 3 - (j & 3) (most significant byte of a u32 word first)
        const uint64_t a0 = desc_start(v) + TG_PAD;
        for (uint32_t q = 0; q * 8 < nbytes; ++q) {
            const uint64_t win = window64(packed, a0 + 32ull * q);
            for (uint32_t t = 0; t < 8 && q * 8 + t < nbytes; ++t) {
                const unsigned long long j = p + q * 8 + t;
                out_bytes[(j & ~3ull) + 3 - (j & 3)] = (uint8_t)(win >> (56 - 8 * t));
            }
        }
    }
}

__global__ void k_rebase(uint64_t* __restrict__ desc, uint64_t n, uint64_t add) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        desc[i] += add;
}

}  // namespace

cudaError_t launch_spill_size(const uint64_t* desc, uint64_t desc_cap, const uint32_t* n_desc, uint32_t n_lists,
                              int k, int shift, uint32_t nb, unsigned long long* totals, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(totals, 0, 16 * (size_t)nb, st);
    if (e != cudaSuccess || !n_lists) return e;
    k_spill_size<<<n_lists, SPILL_THREADS, 0, st>>>(desc, desc_cap, n_desc, k, shift, nb, totals);
    return cudaGetLastError();
}

cudaError_t launch_spill_write(const uint32_t* packed, const uint64_t* desc, uint64_t desc_cap, const uint32_t* n_desc,
                               uint32_t n_lists, int k, int shift, uint32_t nb, unsigned long long* cursors,
                               const long long* host_shift, uint64_t* out_desc, uint8_t* out_bytes, cudaStream_t st) {
    if (!n_lists) return cudaSuccess;
    k_spill_write<<<n_lists, SPILL_THREADS, 0, st>>>(packed, desc, desc_cap, n_desc, k, shift, nb, cursors, host_shift,
                                                    out_desc, out_bytes);
    return cudaGetLastError();
}

cudaError_t launch_rebase(uint64_t* desc, uint64_t n, uint64_t add, int n_sm, cudaStream_t st) {
    if (!n || !add) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)std::max(n_sm, 1) * 8);
    k_rebase<<<(unsigned)blocks, 256, 0, st>>>(desc, n, add);
    return cudaGetLastError();
}

}  // namespace tg
