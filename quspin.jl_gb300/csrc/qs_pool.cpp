// qs_pool.cpp -- cached device allocations (pool_get / pool_put, qs_internal.h).
//
// A free block is reused for a request of at least 3/4 of its size; blocks
// beyond the cap are freed, largest first.  Each free block keeps an event
// recorded on the stream of its last use, and is handed out again only after
// that event has completed.  cudaMalloc failing with out-of-memory frees the
// whole cache and retries once.
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "qs_internal.h"

namespace qs {

namespace {

struct Block {
    void* p;
    cudaEvent_t done;
};

std::mutex g_pool_mu;
std::multimap<size_t, Block> g_free;   // size -> block
size_t g_cached = 0;
size_t g_cap = 0;

size_t cap_bytes() {
    if (g_cap == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) tot = (size_t)80 << 30;
        g_cap = std::min<size_t>(tot / 10, (size_t)32 << 30);
    }
    return g_cap;
}

void drop(const Block& b) {
    if (b.done) {
        cudaEventSynchronize(b.done);
        cudaEventDestroy(b.done);
    }
    cudaFree(b.p);
}

void free_all_locked() {
    for (auto& kv : g_free) drop(kv.second);
    g_free.clear();
    g_cached = 0;
}

}  // namespace

void* pool_get(size_t bytes) {
    Block b{nullptr, nullptr};
    {
        std::lock_guard<std::mutex> g(g_pool_mu);
        auto it = g_free.lower_bound(bytes);
        if (it != g_free.end() && it->first <= bytes + bytes / 3) {
            b = it->second;
            g_cached -= it->first;
            g_free.erase(it);
        }
    }
    if (b.p) {
        if (b.done) {
            cudaEventSynchronize(b.done);
            cudaEventDestroy(b.done);
        }
        return b.p;
    }
    void* p = nullptr;
    note_device_alloc();
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        {
            std::lock_guard<std::mutex> g(g_pool_mu);
            free_all_locked();
        }
        note_device_alloc();
        e = cudaMalloc(&p, bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(e == cudaErrorMemoryAllocation ? QS_ERR_NOMEM : QS_ERR_CUDA,
                    std::string("device allocation: ") + cudaGetErrorString(e));
    }
    return p;
}

void pool_put(void* p, size_t bytes, cudaStream_t last_use) {
    if (!p) return;
    Block b{p, nullptr};
    if (cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventRecord(b.done, last_use) != cudaSuccess) {
        cudaGetLastError();
        if (b.done) cudaEventDestroy(b.done);
        cudaStreamSynchronize(last_use);
        cudaGetLastError();
        b.done = nullptr;
    }
    std::lock_guard<std::mutex> g(g_pool_mu);
    const size_t cap = cap_bytes();
    if (bytes > cap) {
        drop(b);
        return;
    }
    g_free.emplace(bytes, b);
    g_cached += bytes;
    while (g_cached > cap && !g_free.empty()) {
        auto it = std::prev(g_free.end());
        drop(it->second);
        g_cached -= it->first;
        g_free.erase(it);
    }
}

void* mapped_host_address(void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

void pool_trim() {
    std::lock_guard<std::mutex> g(g_pool_mu);
    free_all_locked();
}

}  // namespace qs
