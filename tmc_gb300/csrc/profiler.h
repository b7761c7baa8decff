// Per-stage device timing with CUDA events on the context's stream -- the counterpart of the
// reference's CTimer stage timings (dmc/CTimer.h:123-190, dmc/DualMarchingCubes.h:144-175).
// Off by default; when on, every named stage records an event pair and the accumulated times can
// be read back through tmc_ctx_profile_read.
#pragma once
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace tmc {

struct Prof {
  bool on = false;
  struct Rec {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  std::map<std::string, std::pair<double, int64_t>> acc;  // ms, count
  std::vector<cudaEvent_t> pool;

  cudaEvent_t ev() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  int begin(const char* name, cudaStream_t st) {
    if (!on) return -1;
    Rec r{name, ev(), ev()};
    cudaEventRecord(r.a, st);
    pending.push_back(r);
    return (int)pending.size() - 1;
  }
  void end(int id, cudaStream_t st) {
    if (id < 0) return;
    cudaEventRecord(pending[id].b, st);
  }
  // after a stream synchronize: fold pending records into the totals
  void collect() {
    for (auto& r : pending) {
      float ms = 0;
      if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
        auto& x = acc[r.name];
        x.first += ms;
        x.second += 1;
      }
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    pending.clear();
  }
  ~Prof() {
    for (auto& r : pending) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// RAII stage scope
struct Stage {
  Prof* p;
  int id;
  cudaStream_t st;
  Stage(Prof* pr, const char* name, cudaStream_t s) : p(pr), id(pr ? pr->begin(name, s) : -1), st(s) {}
  ~Stage() {
    if (p) p->end(id, st);
  }
};

}  // namespace tmc
