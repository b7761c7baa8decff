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

namespace tmc {

// Generic compaction scan of 0/1 flags (one byte each): out[i] = number of set flags before i.
__global__ void __launch_bounds__(kScanThreads) flag_tile_sum_kernel(const uint8_t* flags, int64_t n,
                                                                    unsigned long long* tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  unsigned long long s = 0;
  for (int q = 0; q < kScanItems; q++) {
    const int64_t i = base + (int64_t)q * kScanThreads + threadIdx.x;
    if (i < n) s += flags[i] != 0;
  }
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) flag_offsets_kernel(const uint8_t* flags, int64_t n,
                                                                   const unsigned long long* tile_off, int32_t* out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const int64_t mine = base + (int64_t)threadIdx.x * kScanItems;
  uint8_t f[kScanItems];
  unsigned long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    f[q] = (mine + q < n) ? (flags[mine + q] != 0) : 0;
    s += f[q];
  }
  unsigned long long tot;
  unsigned long long pre = block_exclusive_scan<unsigned long long>(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (mine + q < n) out[mine + q] = (int32_t)pre;
    pre += f[q];
  }
}

int64_t scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

int scan_flags(const uint8_t* flags, int64_t n, int32_t* out, unsigned long long* tile_sums,
               unsigned long long* total, cudaStream_t st) {
  const int64_t tiles = scan_tiles(n);
  if (tiles == 0) {
    cudaMemsetAsync(total, 0, sizeof(unsigned long long), st);
    return 0;
  }
  flag_tile_sum_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(flags, n, tile_sums);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(tile_sums, tiles, total);
  flag_offsets_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(flags, n, tile_sums, out);
  return 3;
}

}  // namespace tmc

namespace tmc {

// Exclusive scan of non-negative int32 values: out[i] = sum of in[0..i).
__global__ void __launch_bounds__(kScanThreads) i32_tile_sum_kernel(const int32_t* in, int64_t n,
                                                                   unsigned long long* tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  unsigned long long s = 0;
  for (int q = 0; q < kScanItems; q++) {
    const int64_t i = base + (int64_t)q * kScanThreads + threadIdx.x;
    if (i < n) s += (unsigned long long)in[i];
  }
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) i32_offsets_kernel(const int32_t* in, int64_t n,
                                                                  const unsigned long long* tile_off, int32_t* out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const int64_t mine = base + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  unsigned long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    v[q] = (mine + q < n) ? in[mine + q] : 0;
    s += (unsigned long long)v[q];
  }
  unsigned long long tot;
  unsigned long long pre = block_exclusive_scan<unsigned long long>(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int q = 0; q < kScanItems; q++) {
    if (mine + q < n) out[mine + q] = (int32_t)pre;
    pre += (unsigned long long)v[q];
  }
}

int scan_i32(const int32_t* in, int64_t n, int32_t* out, unsigned long long* tile_sums, unsigned long long* total,
             cudaStream_t st) {
  const int64_t tiles = scan_tiles(n);
  if (tiles == 0) {
    cudaMemsetAsync(total, 0, sizeof(unsigned long long), st);
    return 0;
  }
  i32_tile_sum_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, tile_sums);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(tile_sums, tiles, total);
  i32_offsets_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, tile_sums, out);
  return 3;
}

}  // namespace tmc
