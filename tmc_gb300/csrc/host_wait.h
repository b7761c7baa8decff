// Host waits that sleep.  cudaStreamSynchronize spins a core for the whole wait (the default
// scheduling of a context that has fewer threads than cores); a caller with several extractions
// in flight, or a request server, has many threads waiting at once, and their spinning takes the
// host's cores from the threads that have work.  A blocking-sync event (one per thread and device)
// puts the waiting thread to sleep instead.
#pragma once
#include <vector>
#include <cuda_runtime.h>

namespace tmc {

// Waits for the work queued on `st` so far.  The event belongs to the current device; when it
// cannot be recorded on `st` (a stream of another device, or an event left from before a device
// reset, which is replaced once) the wait falls back to cudaStreamSynchronize.
inline cudaError_t host_wait(cudaStream_t st) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return cudaStreamSynchronize(st);
  }
  thread_local std::vector<cudaEvent_t> events;  // by device
  if ((int)events.size() <= dev) events.resize(dev + 1, nullptr);
  for (int attempt = 0; attempt < 2; attempt++) {
    if (!events[dev] &&
        cudaEventCreateWithFlags(&events[dev], cudaEventBlockingSync | cudaEventDisableTiming) != cudaSuccess) {
      (void)cudaGetLastError();
      events[dev] = nullptr;
      break;
    }
    if (cudaEventRecord(events[dev], st) == cudaSuccess) return cudaEventSynchronize(events[dev]);
    (void)cudaGetLastError();
    events[dev] = nullptr;
  }
  return cudaStreamSynchronize(st);
}

}  // namespace tmc
