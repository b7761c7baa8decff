// Access to a context's device, stream, error message and launch counter for C entry points that
// live outside runtime.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tmc_gb300.h"

#include <map>
#include <mutex>

namespace tmc {
// Pinned host blocks for results copied to host memory (TMC_OUT_HOST), reused across calls by
// power-of-two size class (from 4 KiB), so that varied request sizes still reuse blocks; a class
// met for the first time costs a cudaMallocHost.  Thread-safe: the worker contexts of a request
// server share one pool, so a size class warmed by any of them serves all.
struct PinnedPool {
  std::mutex m;
  std::multimap<size_t, void*> free_blocks;
  std::map<void*, size_t> size_of;
  void* get(size_t bytes) {
    size_t cls = 4096;
    while (cls < bytes) cls <<= 1;
    std::lock_guard<std::mutex> lk(m);
    auto it = free_blocks.lower_bound(cls);
    if (it != free_blocks.end() && it->first <= 2 * cls) {
      void* p = it->second;
      free_blocks.erase(it);
      return p;
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, cls) != cudaSuccess) return nullptr;
    size_of[p] = cls;
    return p;
  }
  void put(void* p) {
    std::lock_guard<std::mutex> lk(m);
    auto it = size_of.find(p);
    if (it != size_of.end()) free_blocks.emplace(it->second, p);
  }
  ~PinnedPool() {
    for (auto& kv : size_of) cudaFreeHost(kv.first);
  }
};

int ctx_device(const tmc_ctx* ctx);
cudaStream_t ctx_stream(const tmc_ctx* ctx);
// stores msg as the context's last error and returns s
tmc_status ctx_fail(tmc_ctx* ctx, tmc_status s, const char* msg);
void ctx_count_launches(tmc_ctx* ctx, int64_t n);
// ctx takes over from's pinned block pool (both must live on the same device)
void ctx_share_pinned(tmc_ctx* ctx, tmc_ctx* from);
}  // namespace tmc
