// Device memory of the library's buffers, kept for reuse.
//
// A context allocates its buffers once (mesh tables, the level store, the merged
// planes, the inverses and the march scratch: ~50 GB for the 4614-DOF sphere) and
// releases them when it is destroyed.  cudaMalloc and cudaFree of buffers that size
// cost milliseconds each (page mapping and unmapping; a context's close measured
// 14 ms), which a caller that creates a context per solve pays on every solve.  Freed
// blocks are therefore kept, keyed by device and rounded size, and handed to the next
// allocation of the same size: a context for a mesh of the same size allocates and
// frees nothing.  The cache holds at most half of the device's memory; a cudaMalloc
// that fails releases the device's cached blocks and tries once more, and
// tdbem_release_cached_memory gives them back on request.
//
// A block may still be read or written by work in flight on the freeing context's
// streams when it is freed: mem_free synchronises the device before the block can be
// handed out again (as cudaFree does implicitly).
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <unordered_map>
#include <utility>
#include <vector>

#include "capi_common.cuh"

namespace tdbem {

namespace {

constexpr int kMaxDevices = 64;

struct MemCache {
    std::mutex mu;
    std::unordered_map<void*, std::pair<int, size_t>> live;  // block -> (device, size)
    std::multimap<std::pair<int, size_t>, void*> kept;       // (device, size) -> block
    size_t kept_bytes[kMaxDevices] = {};
    size_t cap[kMaxDevices] = {};
};

MemCache& cache() {
    static MemCache* c = new MemCache;  // never destroyed: blocks outlive static teardown
    return *c;
}

// Large blocks in 2 MiB steps (so buffers that differ by a few bytes share a size),
// small ones in 512-byte steps.
size_t round_size(size_t bytes) {
    if (bytes == 0) bytes = 1;
    const size_t step = bytes >= (1u << 20) ? (2u << 20) : 512u;
    return (bytes + step - 1) / step * step;
}

}  // namespace

cudaError_t mem_alloc(void** p, size_t bytes) {
    *p = nullptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    const size_t size = round_size(bytes);
    MemCache& c = cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.kept.find({dev, size});
        if (it != c.kept.end()) {
            *p = it->second;
            c.kept.erase(it);
            c.kept_bytes[dev] -= size;
            c.live[*p] = {dev, size};
            return cudaSuccess;
        }
    }
    e = cudaMalloc(p, size);
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();
        mem_release(dev);
        e = cudaMalloc(p, size);
    }
    if (e != cudaSuccess) {
        *p = nullptr;
        return e;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    c.live[*p] = {dev, size};
    return cudaSuccess;
}

void mem_free(void* p) {
    if (!p) return;
    MemCache& c = cache();
    std::pair<int, size_t> key;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.live.find(p);
        if (it == c.live.end()) {  // not from mem_alloc
            cudaFree(p);
            return;
        }
        key = it->second;
        c.live.erase(it);
    }
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != key.first) cudaSetDevice(key.first);
    // work in flight may still use the block
    const cudaError_t es = cudaDeviceSynchronize();
    size_t cap = 0;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        if (!c.cap[key.first]) {
            size_t fr = 0, total = 0;
            if (cudaMemGetInfo(&fr, &total) == cudaSuccess) c.cap[key.first] = total / 2;
        }
        cap = c.cap[key.first];
        if (es == cudaSuccess && c.kept_bytes[key.first] + key.second <= cap) {
            c.kept.insert({key, p});
            c.kept_bytes[key.first] += key.second;
            p = nullptr;
        }
    }
    if (p) cudaFree(p);  // over the cap, or the device reported an error
    if (cur != key.first) cudaSetDevice(cur);
}

size_t mem_release(int device) {
    MemCache& c = cache();
    std::vector<std::pair<int, void*>> out;
    size_t bytes = 0;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        for (auto it = c.kept.begin(); it != c.kept.end();) {
            if (device < 0 || it->first.first == device) {
                out.push_back({it->first.first, it->second});
                bytes += it->first.second;
                c.kept_bytes[it->first.first] -= it->first.second;
                it = c.kept.erase(it);
            } else {
                ++it;
            }
        }
    }
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& b : out) {
        if (b.first != cur) cudaSetDevice(b.first);
        cudaFree(b.second);
        if (b.first != cur) cudaSetDevice(cur);
    }
    return bytes;
}

size_t mem_cached_bytes(int device) {
    MemCache& c = cache();
    std::lock_guard<std::mutex> lk(c.mu);
    if (device >= 0) return device < kMaxDevices ? c.kept_bytes[device] : 0;
    size_t b = 0;
    for (size_t x : c.kept_bytes) b += x;
    return b;
}

}  // namespace tdbem

extern "C" {

int tdbem_cached_memory(int device, size_t* bytes) {
    if (!bytes) return tdbem::capi::fail(TDBEM_ERR_ARG, "bytes is null");
    *bytes = tdbem::mem_cached_bytes(device);
    return TDBEM_OK;
}

int tdbem_release_cached_memory(int device, size_t* released) {
    const size_t b = tdbem::mem_release(device);
    if (released) *released = b;
    return TDBEM_OK;
}

}  // extern "C"
