// Host waits that sleep.  cudaStreamSynchronize spins a core for the whole wait (the default
// scheduling of a context that has fewer threads than cores); a caller with several extractions
// in flight, or a request server, has many threads waiting at once, and their spinning takes the
// host's cores from the threads that have work.  A blocking-sync event (one per thread and device)
// puts the waiting thread to sleep instead.
#pragma once
#include <vector>
#include <cuda_runtime.h>

namespace tmc {

// Waits for the work queued on `st` so far (the stream's device must be the current device).
inline cudaError_t host_wait(cudaStream_t st) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  thread_local std::vector<cudaEvent_t> events;  // by device
  if ((int)events.size() <= dev) events.resize(dev + 1, nullptr);
  for (int attempt = 0; attempt < 2; attempt++) {
    if (!events[dev] &&
        (e = cudaEventCreateWithFlags(&events[dev], cudaEventBlockingSync | cudaEventDisableTiming)) != cudaSuccess) {
      events[dev] = nullptr;
      return e;
    }
    e = cudaEventRecord(events[dev], st);
    if (e == cudaSuccess) return cudaEventSynchronize(events[dev]);
    // an event left from before a device reset: make a new one, once
    (void)cudaGetLastError();
    events[dev] = nullptr;
  }
  return e;
}

}  // namespace tmc
