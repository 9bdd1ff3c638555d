// tg_format.cu — output formatting on the device: counted (k-mer, count)
// pairs to the bytes of tuna's output files.
//
//  TSV  "<kmer>\t<count>\n" per pair, upper-case label, decimal count
//       (write_counts, src/count.hpp:180-216; Kmer::get_label, Kmer.hpp:664-682)
//  KFF  the raw-section entries written through kff-cpp-api
//       (write_counts_kff, src/count.hpp:224-265, src/kff_output.hpp:42-57):
//       ceil(k/4) bytes of 2-bit codes A0 C1 G2 T3, first base in the two high
//       bits of byte 0, last byte padded with zero bits, then the count as 4
//       bytes big-endian (Kmer::write_packed_2bit_msb, Kmer.hpp:685-693)
//  RAW  the key words (little-endian u64, tuna::Kmer<k> layout) then the u32
//       count, packed
//
// A CTA formats a tile of 256 pairs into shared memory (one thread per pair,
// intra-tile offsets from a block scan of the record lengths) and writes the
// tile's bytes with 16-byte stores. TSV records vary in length with the digits
// of the count, so a first kernel sums each tile and a scan gives the tiles'
// offsets; KFF and RAW records have a fixed size.
#include "tg_launch.h"

namespace tg {
namespace {

constexpr int FMT_T = 256;                   // pairs per tile, threads per CTA
constexpr int FMT_MAX_REC = 63 + 2 + 10;     // longest TSV record (k = 63, 10-digit count)

__device__ __forceinline__ uint32_t dec_digits(uint32_t c) {
    uint32_t d = 1;
    for (uint64_t p = 10; c >= p; p *= 10) ++d;  // at most 10 digits
    return d;
}

__device__ __forceinline__ uint32_t rec_len(int fmt, int k, int W, uint32_t count) {
    if (fmt == TG_FMT_TSV) return (uint32_t)k + 2 + dec_digits(count);
    if (fmt == TG_FMT_KFF) return (uint32_t)(k + 3) / 4 + 4;
    return 8u * W + 4;
}

// the 2k-bit code of a key, first base in the high bits of hi:lo (128 bits)
template <int W>
__device__ __forceinline__ void key_msb(const uint64_t* __restrict__ keys, uint64_t i, int k, uint64_t& hi,
                                        uint64_t& lo) {
    if (W == 1) {
        hi = keys[i] << (64 - 2 * k);
        lo = 0;
    } else {
        // word 0: the last 32 bases; word 1: the first k - 32 in its low bits
        const uint64_t w0 = keys[2 * i], w1 = keys[2 * i + 1];
        const int s = 128 - 2 * k;  // 2..64
        if (s == 64) {
            hi = w0;
            lo = 0;
        } else {
            hi = (w1 << s) | (w0 >> (64 - s));
            lo = w0 << s;
        }
    }
}

__global__ void __launch_bounds__(FMT_T) k_fmt_tile_len(const uint32_t* __restrict__ counts, uint64_t n, int k,
                                                        uint32_t* __restrict__ tile_len) {
    __shared__ uint32_t s_sum[FMT_T / 32];
    const uint64_t n_tiles = (n + FMT_T - 1) / FMT_T;
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const uint64_t i = t * FMT_T + threadIdx.x;
        uint32_t len = i < n ? (uint32_t)k + 2 + dec_digits(counts[i]) : 0;
#pragma unroll
        for (int o = 16; o; o >>= 1) len += __shfl_down_sync(~0u, len, o);
        if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = len;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t s = 0;
            for (int w = 0; w < FMT_T / 32; ++w) s += s_sum[w];
            tile_len[t] = s;
        }
        __syncthreads();
    }
}

template <int FMT, int W>
__global__ void __launch_bounds__(FMT_T) k_fmt(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ counts,
                                               uint64_t n, int k, const unsigned long long* __restrict__ tile_off,
                                               uint8_t* __restrict__ out) {
    __shared__ __align__(16) uint8_t s_buf[FMT_T * FMT_MAX_REC + 32];
    __shared__ uint32_t s_warp[FMT_T / 32];
    __shared__ uint32_t s_lut[256];  // 4 codes (first base high) -> 4 letters, first letter in byte 0
    for (int v = threadIdx.x; v < 256; v += FMT_T) {
        uint32_t s = 0;
        for (int j = 0; j < 4; ++j) s |= (uint32_t)("ACGT"[(v >> (6 - 2 * j)) & 3]) << (8 * j);
        s_lut[v] = s;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t n_tiles = (n + FMT_T - 1) / FMT_T;
    for (uint64_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
        const uint64_t i = t * FMT_T + threadIdx.x;
        const bool have = i < n;
        const uint32_t cnt = have ? counts[i] : 0;
        const uint32_t len = have ? rec_len(FMT, k, W, cnt) : 0;
        // exclusive scan of the record lengths over the tile
        uint32_t x = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(~0u, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t wbase = 0, total = 0;
#pragma unroll
        for (int w = 0; w < FMT_T / 32; ++w) {
            const uint32_t v = s_warp[w];
            if (w < warp) wbase += v;
            total += v;
        }
        const unsigned long long g0 =
            FMT == TG_FMT_TSV ? tile_off[t] : (unsigned long long)t * FMT_T * rec_len(FMT, k, W, 1);
        const uint32_t sh = (uint32_t)(((uintptr_t)out + g0) & 15u);
        uint8_t* o = s_buf + sh + wbase + x - len;
        if (have) {
            if (FMT == TG_FMT_RAW) {
                for (int q = 0; q < W; ++q) {
                    const uint64_t v = keys[W * i + q];
                    for (int b = 0; b < 8; ++b) o[8 * q + b] = (uint8_t)(v >> (8 * b));
                }
                for (int b = 0; b < 4; ++b) o[8 * W + b] = (uint8_t)(cnt >> (8 * b));
            } else {
                uint64_t hi, lo;
                key_msb<W>(keys, i, k, hi, lo);
                if (FMT == TG_FMT_KFF) {
                    const int kb = (k + 3) / 4;
                    for (int b = 0; b < kb; ++b) {
                        o[b] = (uint8_t)(hi >> 56);
                        hi = (hi << 8) | (lo >> 56);
                        lo <<= 8;
                    }
                    o[kb] = (uint8_t)(cnt >> 24);
                    o[kb + 1] = (uint8_t)(cnt >> 16);
                    o[kb + 2] = (uint8_t)(cnt >> 8);
                    o[kb + 3] = (uint8_t)cnt;
                } else {
                    for (int b = 0; b < k; b += 4) {
                        const uint32_t four = s_lut[hi >> 56];
                        const int m = min(4, k - b);
                        for (int j = 0; j < m; ++j) o[b + j] = (uint8_t)(four >> (8 * j));
                        hi = (hi << 8) | (lo >> 56);
                        lo <<= 8;
                    }
                    o[k] = '\t';
                    const uint32_t d = len - (uint32_t)k - 2;
                    uint32_t c = cnt;
                    for (int j = (int)d - 1; j >= 0; --j) {
                        o[k + 1 + j] = (uint8_t)('0' + c % 10);
                        c /= 10;
                    }
                    o[k + 1 + d] = '\n';
                }
            }
        }
        __syncthreads();
        // the tile's bytes [g0, g0 + total) with 16-byte stores
        const long long a0 = (long long)g0 - (long long)sh;
        const long long end = (long long)(g0 + total);
        const uint32_t n16 = (uint32_t)((end - a0 + 15) / 16);
        for (uint32_t u = threadIdx.x; u < n16; u += FMT_T) {
            const long long ga = a0 + 16ll * u;
            if (ga >= (long long)g0 && ga + 16 <= end) {
                *reinterpret_cast<uint4*>(out + ga) = *reinterpret_cast<const uint4*>(s_buf + 16 * u);
            } else {
                for (int b = 0; b < 16; ++b) {
                    const long long g = ga + b;
                    if (g >= (long long)g0 && g < end) out[g] = s_buf[16 * u + b];
                }
            }
        }
        __syncthreads();
    }
}

template <int FMT>
cudaError_t launch_fmt_w(int W, const uint64_t* keys, const uint32_t* counts, uint64_t n, int k,
                         const unsigned long long* tile_off, uint8_t* out, unsigned grid, cudaStream_t st) {
    if (W == 1) k_fmt<FMT, 1><<<grid, FMT_T, 0, st>>>(keys, counts, n, k, tile_off, out);
    else k_fmt<FMT, 2><<<grid, FMT_T, 0, st>>>(keys, counts, n, k, tile_off, out);
    return cudaGetLastError();
}

// Digest of pairs [0, n): each thread sums the terms of its pairs, a warp
// reduces them, one atomic per warp and field. out[4] = pairs, count sum, h1,
// h2 (zeroed by the caller).
__global__ void __launch_bounds__(256) k_digest(const uint64_t* __restrict__ keys, int W, int nw,
                                                const uint32_t* __restrict__ counts, uint64_t n,
                                                unsigned long long* __restrict__ out) {
    unsigned long long h1 = 0, h2 = 0, cs = 0, np = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t w0 = keys[i * W];
        const uint64_t w1 = W > 1 ? keys[i * W + 1] : 0;
        const uint32_t c = counts[i];
        uint64_t a, b;
        digest_terms(w0, w1, nw, c, a, b);
        h1 += a;
        h2 += b;
        cs += c;
        ++np;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        h1 += __shfl_down_sync(0xffffffffu, h1, o);
        h2 += __shfl_down_sync(0xffffffffu, h2, o);
        cs += __shfl_down_sync(0xffffffffu, cs, o);
        np += __shfl_down_sync(0xffffffffu, np, o);
    }
    if ((threadIdx.x & 31) == 0 && np) {
        atomicAdd(&out[0], np);
        atomicAdd(&out[1], cs);
        atomicAdd(&out[2], h1);
        atomicAdd(&out[3], h2);
    }
}

}  // namespace

cudaError_t launch_digest(int k, const uint64_t* keys, const uint32_t* counts, uint64_t n, unsigned long long* out,
                          int n_sm, cudaStream_t st, int* launches) {
    const int W = k <= 31 ? 1 : 2;
    const int nw = (k + 31) / 32;
    cudaError_t e = cudaMemsetAsync(out, 0, 4 * sizeof(unsigned long long), st);
    if (e != cudaSuccess || n == 0) return e;
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)std::max(n_sm, 1) * 8);
    k_digest<<<(unsigned)blocks, 256, 0, st>>>(keys, W, nw, counts, n, out);
    ++*launches;
    return cudaGetLastError();
}

size_t fmt_scratch_bytes(uint64_t n_pairs) {
    const uint64_t n_tiles = (n_pairs + FMT_T - 1) / FMT_T;
    return 512 + n_tiles * 4 + (n_tiles + 1) * 8 + 64 * 8 + 3 * 256;
}

uint64_t fmt_max_bytes(int fmt, int k, uint64_t n_pairs) {
    const int W = k <= 31 ? 1 : 2;
    if (fmt == TG_FMT_TSV) return n_pairs * (uint64_t)(k + 12);
    if (fmt == TG_FMT_KFF) return n_pairs * (uint64_t)((k + 3) / 4 + 4);
    return n_pairs * (uint64_t)(8 * W + 4);
}

cudaError_t launch_format(int fmt, int k, const uint64_t* keys, const uint32_t* counts, uint64_t n, uint8_t* out,
                          void* scratch, int n_sm, cudaStream_t st, unsigned long long* d_total, int* launches) {
    const int W = k <= 31 ? 1 : 2;
    const uint64_t n_tiles = (n + FMT_T - 1) / FMT_T;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(n_tiles, (uint64_t)n_sm * 8));
    uint8_t* p = static_cast<uint8_t*>(scratch);
    auto take = [&](size_t bytes) {
        uint8_t* r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    uint32_t* tile_len = reinterpret_cast<uint32_t*>(take(n_tiles * 4 + 4));
    unsigned long long* tile_off = reinterpret_cast<unsigned long long*>(take((n_tiles + 1) * 8));
    unsigned long long* sums = reinterpret_cast<unsigned long long*>(take(64 * 8));
    cudaError_t e = cudaSuccess;
    if (n == 0) return cudaSuccess;
    if (fmt == TG_FMT_TSV) {
        k_fmt_tile_len<<<grid, FMT_T, 0, st>>>(counts, n, k, tile_len);
        ++*launches;
        e = launch_scan(tile_len, n_tiles, tile_off, sums, d_total, st, launches);
        if (e != cudaSuccess) return e;
        e = launch_fmt_w<TG_FMT_TSV>(W, keys, counts, n, k, tile_off, out, grid, st);
    } else {  // fixed record size: the caller knows the total (fmt_max_bytes)
        e = fmt == TG_FMT_KFF ? launch_fmt_w<TG_FMT_KFF>(W, keys, counts, n, k, nullptr, out, grid, st)
                              : launch_fmt_w<TG_FMT_RAW>(W, keys, counts, n, k, nullptr, out, grid, st);
    }
    ++*launches;
    return e;
}

}  // namespace tg
