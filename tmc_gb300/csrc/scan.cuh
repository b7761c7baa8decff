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

// Striped in-tile exclusive scan: warp w of the block owns the tile's cells 256w .. 256w + 255, in
// kScanItems rounds of 32 consecutive cells (lane l takes cell 256w + 32s + l in round s), so that
// the loads of the values and the stores of the offsets are coalesced.  v[s] is the lane's value in
// round s; on return v[s] holds its exclusive prefix within the tile (plus `base`).
__device__ __forceinline__ void tile_striped_exclusive_scan(unsigned long long v[kScanItems],
                                                            unsigned long long base) {
  __shared__ unsigned long long wsum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long run = 0;
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    unsigned long long x = v[s];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const unsigned long long tot = __shfl_sync(0xffffffffu, x, 31);
    v[s] = run + x - v[s];
    run += tot;
  }
  if (lane == 0) wsum[w] = run;
  __syncthreads();
  unsigned long long pre = base;
  for (int q = 0; q < w; q++) pre += wsum[q];
#pragma unroll
  for (int s = 0; s < kScanItems; s++) v[s] += pre;
  __syncthreads();  // wsum is reused by the block's next tile
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
