// Listing the cells of a scan tile that the isosurface crosses (the classification front end shared
// by DMC and TMC): their MC cases from warp-wide ballots, and their slots in cell order (CellMask,
// common.cuh).
#pragma once
#include "common.cuh"
#include "scan.cuh"

namespace tmc {

static_assert(kScanTile == 1 << kTileShift, "listed-cell slots assume 2048-cell scan tiles");

// MC cases of 32 consecutive cells of a volume, one per lane of a warp (every lane must call it):
// each lane loads the point at its own cell's lower x on the four corner rows (y,z), (y+1,z),
// (y,z+1), (y+1,z+1) -- one coalesced 128-byte load per row for the warp -- and takes the points at
// x+1 from the next lane's ballot bits when that lane holds the next cell of the same row (every lane
// but the last of the warp and the last cell of a row); those few lanes load their x+1 points.
// `valid`: the lane has a cell (i, j, k); invalid lanes return 0.
__device__ __forceinline__ unsigned warp_cases(const Grid& g, bool valid, int i, int j, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t sy = g.nx, sz = (int64_t)g.nx * g.ny;
  const float* p = g.f + (valid ? ((int64_t)k * g.ny + j) * g.nx + i : 0);
  // the next lane holds cell (i + 1, j, k) unless this is the warp's last lane or the row's last cell;
  // those lanes load their x+1 points together with the others' loads (no second round trip)
  const bool own_next = valid && (lane == 31 || i >= g.nx - 2);
  bool b0 = false, b1 = false, b2 = false, b3 = false, n0 = false, n1 = false, n2 = false, n3 = false;
  if (valid) {
    b0 = __ldg(p) >= g.iso_up;
    b1 = __ldg(p + sy) >= g.iso_up;
    b2 = __ldg(p + sz) >= g.iso_up;
    b3 = __ldg(p + sz + sy) >= g.iso_up;
  }
  if (own_next) {
    n0 = __ldg(p + 1) >= g.iso_up;
    n1 = __ldg(p + sy + 1) >= g.iso_up;
    n2 = __ldg(p + sz + 1) >= g.iso_up;
    n3 = __ldg(p + sz + sy + 1) >= g.iso_up;
  }
  const unsigned m0 = __ballot_sync(0xffffffffu, b0), m1 = __ballot_sync(0xffffffffu, b1),
                 m2 = __ballot_sync(0xffffffffu, b2), m3 = __ballot_sync(0xffffffffu, b3);
  if (!valid) return 0;
  if (!own_next) {
    n0 = (m0 >> (lane + 1)) & 1u;
    n1 = (m1 >> (lane + 1)) & 1u;
    n2 = (m2 >> (lane + 1)) & 1u;
    n3 = (m3 >> (lane + 1)) & 1u;
  }
  return (unsigned)b0 | (unsigned)n0 << 1 | (unsigned)b1 << 2 | (unsigned)n1 << 3 | (unsigned)b2 << 4 |
         (unsigned)n2 << 5 | (unsigned)b3 << 6 | (unsigned)n3 << 7;
}

// Tile-wide listing of the cells whose `act` bit is set, in cell order: each warp's ballot masks of
// the tile's 64 words (word = s * 8 + warp: step s of the blocked loop covers offsets s * 256 .. +255)
// are scanned by one warp; the words with their in-tile prefixes go to `mask` (CellMask per 32
// cells), the listed offsets to `list`.  Returns the tile's listed count.  Every thread calls it.
__device__ __forceinline__ int list_tile(unsigned actbits, int64_t tile, CellMask* mask, uint32_t* wmask,
                                         uint32_t* wpre, uint16_t* list, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int kWords = kScanTile / 32;  // 64
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    const unsigned bal = __ballot_sync(0xffffffffu, (actbits >> s) & 1u);
    if (lane == 0) wmask[s * (kScanThreads / 32) + wid] = bal;
  }
  __syncthreads();
  if (wid == 0) {
    const uint32_t a = wmask[2 * lane], b = wmask[2 * lane + 1];
    const int ca = __popc(a), cb = __popc(b);
    int x = ca + cb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const int ex = x - ca - cb;
    wpre[2 * lane] = (uint32_t)ex;
    wpre[2 * lane + 1] = (uint32_t)(ex + ca);
    uint4* m = reinterpret_cast<uint4*>(mask + tile * kWords) + lane;  // 16-byte store of two words
    *m = make_uint4(a, (uint32_t)ex, b, (uint32_t)(ex + ca));
    if (lane == 31) *total = x;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int s = 0; s < kScanItems; s++)
    if ((actbits >> s) & 1u) {
      const int w = s * (kScanThreads / 32) + wid;
      list[wpre[w] + __popc(wmask[w] & lt)] = (uint16_t)(s * kScanThreads + threadIdx.x);
    }
  __syncthreads();
  return *total;
}

}  // namespace tmc
