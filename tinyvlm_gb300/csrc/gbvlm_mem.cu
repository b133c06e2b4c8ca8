// Device and pinned host memory for plans that are created and destroyed
// while other streams keep the GPU busy (the served mode creates a batched
// plan per admitted request group).  cudaMalloc and cudaFree synchronise the
// whole device, so a plan released by one lane would wait for every other
// lane's work in flight; stream-ordered allocations from the device's
// default memory pool do not.
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <vector>

#include "gbvlm_internal.h"

namespace gbvlm {

namespace {

std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;

cudaMemPool_t default_pool(cudaError_t* err) {
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> g(g_pool_mu);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) return it->second;
    cudaMemPool_t p = nullptr;
    *err = cudaDeviceGetDefaultMemPool(&p, dev);
    if (*err != cudaSuccess) return nullptr;
    // keep freed blocks in the pool for the next plan (a process-local
    // attribute of this process's pool)
    uint64_t keep = UINT64_MAX;
    *err = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (*err != cudaSuccess) return nullptr;
    g_pools[dev] = p;
    return p;
}

std::mutex g_pin_mu;
std::map<size_t, std::vector<void*>> g_pinned;  // free blocks by size class

size_t size_class(size_t bytes) {
    size_t c = 256;
    while (c < bytes) c <<= 1;
    return c;
}

}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t mem) {
    *p = nullptr;
    if (!mem) return cudaMalloc(p, bytes);
    cudaError_t e = cudaSuccess;
    cudaMemPool_t pool = default_pool(&e);
    if (!pool) return e;
    e = cudaMallocFromPoolAsync(p, bytes, pool, mem);
    // `mem` carries nothing else while a plan is built: this returns once the
    // block is usable on every stream
    if (e == cudaSuccess) e = cudaStreamSynchronize(mem);
    return e;
}

void dev_free(void* p, cudaStream_t mem) {
    if (!p) return;
    if (mem)
        cudaFreeAsync(p, mem);
    else
        cudaFree(p);
}

void* pinned_take(size_t bytes) {
    const size_t c = size_class(bytes);
    {
        std::lock_guard<std::mutex> g(g_pin_mu);
        auto& v = g_pinned[c];
        if (!v.empty()) {
            void* p = v.back();
            v.pop_back();
            return p;
        }
    }
    void* p = nullptr;
    return cudaMallocHost(&p, c) == cudaSuccess ? p : nullptr;
}

void pinned_give(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> g(g_pin_mu);
    g_pinned[size_class(bytes)].push_back(p);
}

}  // namespace gbvlm
