#include "scan.cuh"

namespace tmc {

// One block of 1024 threads scans all tile sums: each thread owns a contiguous chunk.
__global__ void scan_tile_sums_kernel(unsigned long long* sums, int64_t ntiles, unsigned long long* totals) {
  constexpr int T = 1024;
  __shared__ unsigned long long part[T];
  const int tid = threadIdx.x;
  const int64_t per = (ntiles + T - 1) / T;
  const int64_t b = tid * per, e = b + per < ntiles ? b + per : ntiles;
  unsigned long long s = 0;
  for (int64_t i = b; i < e; i++) s += sums[i];
  part[tid] = s;
  __syncthreads();
  // Hillis-Steele over 1024 partial sums
  for (int o = 1; o < T; o <<= 1) {
    unsigned long long y = (tid >= o) ? part[tid - o] : 0ull;
    __syncthreads();
    part[tid] += y;
    __syncthreads();
  }
  unsigned long long run = tid ? part[tid - 1] : 0ull;
  for (int64_t i = b; i < e; i++) {
    const unsigned long long v = sums[i];
    sums[i] = run;
    run += v;
  }
  if (tid == T - 1) totals[0] = part[T - 1];
}

}  // namespace tmc
