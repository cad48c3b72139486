// nf_alloc.cu -- the device-memory cache of the library's buffers.
//
// A handle sizes its buffers on the fly (rounds grow them), and a batch of
// hundreds of realisations holds a few GB; cudaMalloc and cudaFree of such
// blocks cost more than the stages that use them when handles come and go
// (one nf_batch_run after another, one plain handle per realisation). Freed
// blocks therefore go to a process-wide cache, per device, with sizes rounded
// up to four classes per power of two (at most 25 % over the request), and a
// request takes the smallest cached block that fits without calling
// cudaMalloc.
// The cache holds at most a quarter of the device's memory (and at most
// 64 GiB); beyond that freed blocks go back to the driver, and
// nf_release_cached_memory() empties it. Returning a block first waits for
// the device (as cudaFree does), so no kernel still in flight on another
// stream can see the block reused.
#include <map>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/nanofiller_gb300.h"
#include "nf_common.cuh"

namespace nf {

namespace {

struct BlockCache {
    std::mutex m;
    // per device: size class bytes -> cached blocks of that class
    std::map<int, std::map<size_t, std::vector<void*>>> free;
    size_t bytes = 0;
};

BlockCache& cache() {
    static BlockCache* c = new BlockCache();  // never destroyed: no CUDA calls at process exit
    return *c;
}

size_t size_class(size_t b) {
    if (b <= 4096) return 4096;
    int e = 63 - __builtin_clzll((unsigned long long)(b - 1));  // 2^e < b <= 2^(e+1)
    const size_t base = (size_t)1 << e, q = base / 4;
    return base + ((b - base + q - 1) / q) * q;
}

size_t cache_limit(int dev) {  // with dev current
    size_t fr = 0, tot = 0;
    (void)dev;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) tot = 0;
    const size_t lim = tot / 4;
    const size_t cap = (size_t)64 << 30;
    return lim < cap ? lim : cap;
}

}  // namespace

cudaError_t dev_alloc(void** p, size_t* bytes) {
    ++g_allocs;  // a request, whether the cache or cudaMalloc serves it
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const size_t cls = size_class(*bytes);
    {
        // best fit: the smallest cached block of at least the request (a
        // buffer that grows round by round then finds the size it will reach);
        // requests below 64 KiB take blocks of at most 1 MiB
        BlockCache& c = cache();
        std::lock_guard<std::mutex> g(c.m);
        auto& bins = c.free[dev];
        for (auto it = bins.lower_bound(cls); it != bins.end(); ++it) {
            if (cls < ((size_t)64 << 10) && it->first > ((size_t)1 << 20)) break;
            if (it->second.empty()) continue;
            *p = it->second.back();
            it->second.pop_back();
            c.bytes -= it->first;
            *bytes = it->first;
            return cudaSuccess;
        }
    }
    e = cudaMalloc(p, cls);
    if (e == cudaErrorMemoryAllocation) {  // give the cached blocks back and try once more
        (void)cudaGetLastError();
        nf_release_cached_memory();
        e = cudaMalloc(p, cls);
    }
    if (e == cudaSuccess) *bytes = cls;
    return e;
}

void dev_free(void* p, size_t bytes) {
    if (!p) return;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { (void)cudaGetLastError(); cudaFree(p); return; }
    const int dev = at.device;  // the block's own device, whichever is current
    const size_t cls = size_class(bytes);  // bytes is a class size already
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != dev) cudaSetDevice(dev);
    cudaDeviceSynchronize();  // no kernel still in flight may see the block reused
    const size_t lim = cache_limit(dev);
    if (cur != dev) cudaSetDevice(cur);
    BlockCache& c = cache();
    {
        std::lock_guard<std::mutex> g(c.m);
        if (c.bytes + cls <= lim) {
            c.free[dev][cls].push_back(p);
            c.bytes += cls;
            return;
        }
    }
    cudaFree(p);
}

}  // namespace nf

extern "C" nf_status nf_release_cached_memory(void) {
    nf::BlockCache& c = nf::cache();
    std::lock_guard<std::mutex> g(c.m);
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& dv : c.free) {
        const int dev = dv.first;
        if (dev != cur) cudaSetDevice(dev);
        for (auto& kv : dv.second) {
            for (void* p : kv.second) cudaFree(p);
            kv.second.clear();
        }
        if (dev != cur) cudaSetDevice(cur);
    }
    c.bytes = 0;
    return NF_OK;
}
