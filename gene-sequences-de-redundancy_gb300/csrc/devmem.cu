// devmem.cu -- the library's stream-ordered device memory pool and pinned
// host slots (devmem.h).
#include "devmem.h"

#include <cstdint>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace gsdr {

namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kPinnedArenaSlots = 64;

std::mutex g_pool_mu;
cudaMemPool_t g_pool[kMaxDevices] = {};
bool g_pool_failed[kMaxDevices] = {};

// The pool of the current device, created on first use: memory freed into it
// is kept for later jobs up to the retained size, and an allocation never
// waits on another stream's work to reuse a block (a block freed on another
// stream is reused only once that free has completed; otherwise the pool grows).
cudaMemPool_t current_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pool[dev] && !g_pool_failed[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
            g_pool_failed[dev] = true;
            return nullptr;
        }
        uint64_t keep = 16384ull << 20;
        if (const char* e = std::getenv("GSDR_POOL_KEEP_MB")) keep = std::strtoull(e, nullptr, 10) << 20;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        int no = 0;
        cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowInternalDependencies, &no);
        g_pool[dev] = p;
    }
    return g_pool[dev];
}

std::mutex g_pin_mu;
std::vector<void*> g_pin_free;

}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    cudaMemPool_t pool = current_pool();
    // without a pool of its own (creation refused) the device's default pool
    // still keeps the allocation stream-ordered
    return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMallocAsync(p, bytes, s);
}

void dev_free(void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

void* pinned_slot() {
    std::lock_guard<std::mutex> lock(g_pin_mu);
    if (g_pin_free.empty()) {
        void* arena = nullptr;
        // portable: usable from every device's context; arenas live until exit
        if (cudaHostAlloc(&arena, kPinnedSlot * kPinnedArenaSlots, cudaHostAllocPortable) !=
            cudaSuccess)
            return nullptr;
        for (size_t i = 0; i < kPinnedArenaSlots; i++)
            g_pin_free.push_back(static_cast<char*>(arena) + i * kPinnedSlot);
    }
    void* p = g_pin_free.back();
    g_pin_free.pop_back();
    std::memset(p, 0, kPinnedSlot);
    return p;
}

void pinned_release(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_pin_mu);
    g_pin_free.push_back(p);
}

namespace {
struct PinnedScratch {
    void* p = nullptr;
    size_t cap = 0;
    ~PinnedScratch() {
        if (p) cudaFreeHost(p);
    }
};
}  // namespace

void* pinned_scratch(size_t bytes) {
    static thread_local PinnedScratch s;
    if (bytes <= s.cap) return s.p;
    if (s.p) cudaFreeHost(s.p);
    s.p = nullptr;
    s.cap = 0;
    const size_t want = std::max(bytes, (size_t)1 << 20);
    if (cudaHostAlloc(&s.p, want, cudaHostAllocPortable) != cudaSuccess) {
        s.p = nullptr;
        return nullptr;
    }
    s.cap = want;
    return s.p;
}

}  // namespace gsdr
