#include "scan.cuh"

namespace tmc {

// One block of 1024 threads scans all tile sums in place.  Warp w owns a contiguous segment of
// 32 * rounds sums and walks it in rounds of 32 consecutive sums (coalesced), carrying its running
// sum; the warps' totals are scanned in shared memory, then each warp writes its exclusive prefixes.
__global__ void scan_tile_sums_kernel(unsigned long long* sums, int64_t ntiles, unsigned long long* totals) {
  constexpr int T = 1024, W = T / 32;
  __shared__ unsigned long long wsum[W];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t rounds = (ntiles + T - 1) / T;
  const int64_t seg = (int64_t)w * 32 * rounds;
  unsigned long long run = 0;
  for (int64_t r = 0; r < rounds; r++) {
    const int64_t i = seg + 32 * r + lane;
    unsigned long long x = i < ntiles ? sums[i] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) wsum[w] = run;
  __syncthreads();
  if (w == 0) {
    unsigned long long x = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    wsum[lane] = x;  // inclusive
  }
  __syncthreads();
  unsigned long long pre = w ? wsum[w - 1] : 0ull;
  for (int64_t r = 0; r < rounds; r++) {
    const int64_t i = seg + 32 * r + lane;
    const unsigned long long v = i < ntiles ? sums[i] : 0ull;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (i < ntiles) sums[i] = pre + x - v;
    pre += __shfl_sync(0xffffffffu, x, 31);
  }
  if (threadIdx.x == T - 1) totals[0] = wsum[W - 1];
}
}  // namespace tmc

namespace tmc {

// Generic compaction scan of 0/1 flags (one byte each): out[i] = number of set flags before i.
__global__ void __launch_bounds__(kScanThreads) flag_tile_sum_kernel(const uint8_t* flags, int64_t n,
                                                                    unsigned long long* tile_sums) {
  uint32_t f[kScanItems];
  load8(flags, (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems, n, f);
  unsigned long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) s += f[q] != 0;
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) flag_offsets_kernel(const uint8_t* flags, int64_t n,
                                                                   const unsigned long long* tile_off, int32_t* out) {
  const int64_t first = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t f[kScanItems];
  load8(flags, first, n, f);
  int32_t sum = 0;
#pragma unroll
  for (int s = 0; s < kScanItems; s++) sum += f[s] != 0;
  int32_t tot;
  int32_t pre = (int32_t)tile_off[blockIdx.x] + block_exclusive_scan(sum, &tot);
  int32_t o[kScanItems];
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    o[s] = pre;
    pre += f[s] != 0;
  }
  store8(out, first, n, o);
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
  uint32_t x[kScanItems];
  load8(reinterpret_cast<const uint32_t*>(in), (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems, n,
        x);
  unsigned long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanItems; q++) s += x[q];
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(s, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) i32_offsets_kernel(const int32_t* in, int64_t n,
                                                                  const unsigned long long* tile_off, int32_t* out) {
  const int64_t first = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t x[kScanItems];
  load8(reinterpret_cast<const uint32_t*>(in), first, n, x);
  unsigned long long sum = 0;
#pragma unroll
  for (int s = 0; s < kScanItems; s++) sum += x[s];
  unsigned long long tot;
  unsigned long long pre = tile_off[blockIdx.x] + block_exclusive_scan(sum, &tot);
  int32_t o[kScanItems];
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    o[s] = (int32_t)pre;
    pre += x[s];
  }
  store8(out, first, n, o);
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
