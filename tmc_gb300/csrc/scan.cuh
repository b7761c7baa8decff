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

// Blocked tile layout: thread t of tile b owns the kScanItems consecutive elements from
// b * kScanTile + t * kScanItems, read and written as 16-byte vectors (contiguous across the warp,
// so the accesses stay coalesced), and scans them serially; one block scan of the thread totals
// then gives every element its offset.  Elements at n and beyond read as 0 and are not written;
// a range that is not 16-byte aligned falls back to scalar accesses.
static_assert(kScanItems == 8, "the blocked accessors move 8 elements per thread");
__device__ __forceinline__ void load8(const uint32_t* p, int64_t first, int64_t n, uint32_t r[8]) {
  const uint32_t* q = p + first;
  if (first + 8 <= n && ((uintptr_t)q & 15) == 0) {
    const uint4 a = *reinterpret_cast<const uint4*>(q), b = *reinterpret_cast<const uint4*>(q + 4);
    r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
    r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
  } else {
#pragma unroll
    for (int s = 0; s < 8; s++) r[s] = first + s < n ? q[s] : 0u;
  }
}
__device__ __forceinline__ void load8(const uint8_t* p, int64_t first, int64_t n, uint32_t r[8]) {
  const uint8_t* q = p + first;
  if (first + 8 <= n && ((uintptr_t)q & 7) == 0) {
    const uint2 a = *reinterpret_cast<const uint2*>(q);
#pragma unroll
    for (int s = 0; s < 4; s++) {
      r[s] = (a.x >> (8 * s)) & 0xffu;
      r[4 + s] = (a.y >> (8 * s)) & 0xffu;
    }
  } else {
#pragma unroll
    for (int s = 0; s < 8; s++) r[s] = first + s < n ? q[s] : 0u;
  }
}
__device__ __forceinline__ void store8(int32_t* p, int64_t first, int64_t n, const int32_t v[8]) {
  int32_t* q = p + first;
  if (first + 8 <= n && ((uintptr_t)q & 15) == 0) {
    *reinterpret_cast<int4*>(q) = make_int4(v[0], v[1], v[2], v[3]);
    *reinterpret_cast<int4*>(q + 4) = make_int4(v[4], v[5], v[6], v[7]);
  } else {
#pragma unroll
    for (int s = 0; s < 8; s++)
      if (first + s < n) q[s] = v[s];
  }
}

// In-tile offsets with one warp per tile: the tile's listed slots are walked 256 at a time, each
// lane owning 8 consecutive slots (the blocked accessors above), scanned with warp shuffles and a
// carry from one step to the next; no block barrier, and a tile's few listed slots (a few hundred
// of its 2048) cost a step or two.
constexpr int kOffsetWarps = 8;  // tiles per block
constexpr int kOffsetStep = 32 * kScanItems;
// inclusive warp scan of a 64-bit value (all lanes of the warp take part)
__device__ __forceinline__ unsigned long long warp_inclusive_scan(unsigned long long x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
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
