// hostmem.cpp — page-locked host memory for the host link (tg_host_alloc).
//
// The CUDA driver's own pinned allocations (cudaHostAlloc, portable to every
// device). On the GB300's Grace host they were measured at the link's rate
// for buffers of tens of GB (H2D ~211 GB/s, D2H ~193 GB/s), where anonymous
// memory mapped with transparent huge pages and registered afterwards
// (cudaHostRegister) fell to ~57 GB/s D2H at 35 GB. The library uses it for its
// own staging buffers; callers use it for the inputs and outputs of the
// one-call entry points. A registry keeps the sizes, so that tg_host_free
// rejects pointers it did not hand out.
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>

#include "tg_host.h"
#include "tuna_gpu.h"

namespace tgh {
namespace {

std::mutex g_mu;
std::unordered_map<void*, size_t>& registry() {
    static std::unordered_map<void*, size_t> m;
    return m;
}

}  // namespace

void* pinned_alloc(size_t bytes, std::string* err) {
    void* p = nullptr;
    const cudaError_t e = cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        if (err) *err = std::string("cudaHostAlloc: ") + cudaGetErrorString(e);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    registry()[p] = bytes;
    return p;
}

bool pinned_free(void* p) {
    if (!p) return true;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = registry().find(p);
        if (it == registry().end()) return false;
        registry().erase(it);
    }
    (void)cudaFreeHost(p);
    (void)cudaGetLastError();
    return true;
}

}  // namespace tgh

extern "C" tg_status tg_host_alloc(size_t bytes, void** out) {
    if (!out) return TG_ERR_ARG;
    *out = nullptr;
    try {
        void* p = tgh::pinned_alloc(bytes, nullptr);
        if (!p) return TG_ERR_OOM;
        *out = p;
        return TG_OK;
    } catch (...) {
        return TG_ERR_OOM;
    }
}

extern "C" tg_status tg_host_free(void* p) {
    try {
        return tgh::pinned_free(p) ? TG_OK : TG_ERR_ARG;
    } catch (...) {
        return TG_ERR_ARG;
    }
}
