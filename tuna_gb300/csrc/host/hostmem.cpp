// hostmem.cpp — page-locked host memory for the host link (tg_host_alloc).
//
// On the GB300's Grace host the copy engines reach host memory through the
// system MMU. Buffers pinned from 4 KiB pages (cudaHostAlloc, a framework's
// pinned allocator) were measured to copy at 9-25 GB/s in some box states,
// where buffers backed by 2 MiB pages copied at the link's ~200 GB/s from the
// first pass. This allocator maps anonymous memory, asks for transparent huge
// pages (madvise MADV_HUGEPAGE; ignored where THP is off), faults the pages in
// from several threads and registers the range with the CUDA runtime
// (portable: usable with every device). The library uses it for its own
// staging buffers; callers use it for the inputs and outputs of the one-call
// entry points.
#include <cuda_runtime.h>
#include <sys/mman.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tg_host.h"
#include "tuna_gpu.h"

namespace tgh {
namespace {

constexpr size_t HUGE = 2u << 20;

std::mutex g_mu;
std::unordered_map<void*, size_t>& registry() {
    static std::unordered_map<void*, size_t> m;
    return m;
}

// First touch of every page, on several threads (each 2 MiB page is one fault
// with THP; one thread would take ~0.3 s per 3 GB).
void prefault(uint8_t* p, size_t len) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::max<size_t>(1, std::min<size_t>(hw, len / (64u << 20)));
    auto body = [p, len, nt](unsigned t) {
        const size_t a = len / HUGE * t / nt * HUGE, b = t + 1 == nt ? len : len / HUGE * (t + 1) / nt * HUGE;
        for (size_t o = a; o < b; o += 4096) p[o] = 0;
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
    for (auto& x : th) x.join();
}

}  // namespace

void* pinned_alloc(size_t bytes, std::string* err) {
    const size_t len = (std::max<size_t>(bytes, 1) + HUGE - 1) / HUGE * HUGE;
    void* p = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (p == MAP_FAILED) {
        if (err) *err = "mmap of " + std::to_string(len) + " bytes failed";
        return nullptr;
    }
    (void)madvise(p, len, MADV_HUGEPAGE);
    prefault(static_cast<uint8_t*>(p), len);
    const cudaError_t e = cudaHostRegister(p, len, cudaHostRegisterPortable);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        munmap(p, len);
        if (err) *err = std::string("cudaHostRegister: ") + cudaGetErrorString(e);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    registry()[p] = len;
    return p;
}

bool pinned_free(void* p) {
    if (!p) return true;
    size_t len = 0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = registry().find(p);
        if (it == registry().end()) return false;
        len = it->second;
        registry().erase(it);
    }
    (void)cudaHostUnregister(p);
    (void)cudaGetLastError();
    munmap(p, len);
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
