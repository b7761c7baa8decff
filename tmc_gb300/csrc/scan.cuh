// Block-level and device-wide exclusive scans used for deterministic compaction: every output
// element gets its index from a prefix sum over cells (or faces, vertices) in grid order, so
// results come out in the same order as the reference's sequential loops.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tmc {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;                              // per thread
constexpr int kScanTile = kScanThreads * kScanItems;       // elements per block

// Exclusive block scan of one value per thread (blockDim.x == kScanThreads).  Returns the
// exclusive prefix; *total receives the block total.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* total) {
  __shared__ T warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    T s = (lane < kScanThreads / 32) ? warp_sums[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const T warp_prefix = wid ? warp_sums[wid - 1] : T(0);
  *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

// Two counters packed in one 64-bit word (high: a, low: b) scan together: both stay far below
// 2^32 per tile, so carries never cross.
struct Pair {
  uint64_t w;
};

// Pass 2 of a device-wide scan: exclusive scan of the per-tile sums in place, in one block.
// sums holds `ntiles` 64-bit packed pairs; totals[0..1] get the grand totals as 64-bit.
__global__ void scan_tile_sums_kernel(unsigned long long* sums, int64_t ntiles, unsigned long long* totals);

// Device-wide compaction scan of byte flags; tile_sums needs scan_tiles(n) words.  Returns the
// number of kernels launched.
int64_t scan_tiles(int64_t n);
int scan_flags(const uint8_t* flags, int64_t n, int32_t* out, unsigned long long* tile_sums,
               unsigned long long* total, cudaStream_t st);
// Device-wide exclusive scan of non-negative int32 values (same tile scheme).
int scan_i32(const int32_t* in, int64_t n, int32_t* out, unsigned long long* tile_sums, unsigned long long* total,
             cudaStream_t st);

}  // namespace tmc
