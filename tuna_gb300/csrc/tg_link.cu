// tg_link.cu — large copies between device memory and page-locked host memory
// done by the SMs (loads and stores through the host buffer's mapped address)
// instead of the copy engines.
//
// Why: on the GB300's Grace host, after another process had churned through a
// few tens of GB of host memory, copy-engine transfers of a freshly pinned
// 24 GB buffer ran at 60-78 GB/s (H2D and D2H) for every repetition, while a
// kernel moving the same bytes through the mapped address kept 181-193 GB/s;
// on a fresh host both ran at the link's 211 GB/s (H2D) and 193 GB/s (D2H).
// Pageable (unregistered) memory, small copies and pairs of pointers that are
// not equally aligned mod 16 keep cudaMemcpyAsync.
#include <cstdint>

#include "tg_launch.h"

namespace tg {
namespace {

constexpr size_t LINK_MIN_BYTES = 1u << 20;

// n bytes from src to dst (either may be mapped host memory); src and dst have
// the same alignment mod 16. k_link_copy moves the 16-byte words between dst's
// first and last 16-byte boundary, k_link_edges the bytes around them. CTAs of
// 256 threads at 32 registers, so that one fits on an SM beside a resident
// counting CTA: the copy of a counting wave's pairs runs while the next wave
// counts.
constexpr int LINK_THREADS = 256;

__global__ void __launch_bounds__(LINK_THREADS, 8) k_link_copy(const uint4* __restrict__ s, uint4* __restrict__ d,
                                                               size_t nv) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < nv; i += 4 * stride) {  // four loads in flight per thread
        const uint4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
        d[i] = a;
        d[i + stride] = b;
        d[i + 2 * stride] = c;
        d[i + 3 * stride] = e;
    }
    for (; i < nv; i += stride) d[i] = s[i];
}

__global__ void k_link_edges(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t head, size_t tail0,
                             size_t n) {
    for (size_t b = threadIdx.x; b < head; b += blockDim.x) dst[b] = src[b];
    for (size_t b = tail0 + threadIdx.x; b < n; b += blockDim.x) dst[b] = src[b];
}

}  // namespace

// The device address of a host pointer when it lies in page-locked memory
// mapped for the current device, else null.
const void* mapped_address(const void* host) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

cudaError_t link_copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st, int n_sm,
                      int* launches) {
    if (bytes >= LINK_MIN_BYTES && (kind == cudaMemcpyHostToDevice || kind == cudaMemcpyDeviceToHost)) {
        const void* s = src;
        void* d = dst;
        if (kind == cudaMemcpyHostToDevice) s = mapped_address(src);
        else d = const_cast<void*>(mapped_address(dst));
        if (s && d && ((reinterpret_cast<uintptr_t>(s) ^ reinterpret_cast<uintptr_t>(d)) & 15) == 0) {
            const uint8_t* s8 = static_cast<const uint8_t*>(s);
            uint8_t* d8 = static_cast<uint8_t*>(d);
            const size_t mis = (16 - (reinterpret_cast<uintptr_t>(d8) & 15)) & 15;
            const size_t head = mis < bytes ? mis : bytes;
            const size_t nv = (bytes - head) / 16, tail0 = head + nv * 16;
            if (nv) {
                const unsigned grid = (unsigned)(n_sm > 0 ? n_sm : 1) * 2;
                k_link_copy<<<grid, LINK_THREADS, 0, st>>>(reinterpret_cast<const uint4*>(s8 + head),
                                                           reinterpret_cast<uint4*>(d8 + head), nv);
                if (launches) ++*launches;
            }
            if (head || tail0 < bytes) {
                k_link_edges<<<1, 32, 0, st>>>(s8, d8, head, tail0, bytes);
                if (launches) ++*launches;
            }
            return cudaGetLastError();
        }
    }
    return bytes ? cudaMemcpyAsync(dst, src, bytes, kind, st) : cudaSuccess;
}

}  // namespace tg
