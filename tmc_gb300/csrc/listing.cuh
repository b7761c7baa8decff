// Listing the cells of a scan tile that the isosurface crosses (the classification front end shared
// by DMC and TMC): their MC cases from warp-wide ballots, and their slots in cell order (CellMask,
// common.cuh).
#pragma once
#include "common.cuh"
#include "generators.cuh"
#include "scan.cuh"

namespace tmc {

static_assert(kScanTile == 1 << kTileShift, "listed-cell slots assume 2048-cell scan tiles");

// Pass 1 of both classifications: the MC case of each of the tile's kScanTile cells (linear order,
// thread t takes cells t, t + 256, ..., so that at each step the 32 lanes of a warp hold 32
// consecutive cells), stored in case_of; returns the thread's listed bits (bit s: the cell of step s
// has a case other than 0 and 255).
//
// Per step each lane loads the point at its cell's lower x on the four corner rows (y,z), (y+1,z),
// (y,z+1), (y+1,z+1) -- one coalesced 128-byte load per row and warp -- and the warp's ballots of the
// comparisons give every lane the bits at x and x+1 at once ((mask >> lane) & 3) when the next lane
// holds the next cell of the same row.  The warp's last lane and a row's last cell load their x+1
// points too, in the same round trip.  Coordinates and the point index advance by 256 cells per step
// (one row wrap at most on rows of 256 cells or more, a division otherwise).
// kGen: the field is generated (Grid::gen) instead of read: every lane evaluates its points, and the
// points whose lower cell it holds (at the upper borders also the border points next to it) are
// written once to Grid::gen_out for the passes that follow.
template <bool kGen = false>
__device__ __forceinline__ unsigned tile_cases(const Grid& g, int64_t space_n, int64_t vbase, uint8_t* case_of) {
  const int lane = threadIdx.x & 31;
  const int64_t n = g.ncells();
  const int cx = g.nx - 1, cy = g.ny - 1;
  const int64_t sy = g.nx, sz = (int64_t)g.nx * g.ny, szy = sz + sy;
  const int64_t c0 = vbase + threadIdx.x - g.vbase;  // the thread's first cell in its volume
  // cells of the volume in this tile, from the thread's first: c0 + 256 s < lim
  const int64_t lim = (space_n - g.vbase < n ? space_n - g.vbase : n);
  int i = 0, j = 0, k = 0;
  if (c0 < lim) {
    const uint32_t cc = (uint32_t)c0;
    const uint32_t r = g.div_cx.div(cc);
    i = (int)(cc - r * (uint32_t)cx);
    const uint32_t kk = g.div_cy.div(r);
    j = (int)(r - kk * (uint32_t)cy);
    k = (int)kk;
  }
  int64_t pi = ((int64_t)k * g.ny + j) * g.nx + i;  // point (i, j, k)
  const float iso = g.iso_up;
  // fused generation: the generator's per-axis tables and kind, read once (the field stores below
  // could otherwise alias them and force a reload per point)
  const float2 *tx = nullptr, *ty = nullptr, *tz = nullptr;
  int surf = 0;
  if (kGen) {
    tx = (const float2*)__ldg((const unsigned long long*)&g.gen->tab[0]);
    ty = (const float2*)__ldg((const unsigned long long*)&g.gen->tab[1]);
    tz = (const float2*)__ldg((const unsigned long long*)&g.gen->tab[2]);
    surf = __ldg(&g.gen->surface);
  }
  unsigned actbits = 0;
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    const bool valid = c0 + (int64_t)s * kScanThreads < lim;
    if (s > 0 && valid) {
      if (cx >= kScanThreads) {
        i += kScanThreads;
        pi += kScanThreads;
        if (i >= cx) {  // next row: skip the row's last point
          i -= cx;
          pi += 1;
          if (++j >= cy) {  // next plane: skip the plane's last row
            j = 0;
            ++k;
            pi += g.nx;
          }
        }
      } else {
        const uint32_t cc = (uint32_t)(c0 + (int64_t)s * kScanThreads);
        const uint32_t r = g.div_cx.div(cc);
        i = (int)(cc - r * (uint32_t)cx);
        const uint32_t kk = g.div_cy.div(r);
        j = (int)(r - kk * (uint32_t)cy);
        k = (int)kk;
        pi = ((int64_t)k * g.ny + j) * g.nx + i;
      }
    }
    const float* p = g.f + pi;
    const bool own_next = valid && (lane == 31 || i == cx - 1);
    bool b0 = false, b1 = false, b2 = false, b3 = false;
    unsigned nx_bits = 0;
    if (kGen) {
      if (valid) {
        const GenParams& P = *g.gen;
        float* o = g.gen_out + pi;
        const bool lj = j == cy - 1, lk = k == g.nz - 2;  // the cell touches the upper y / z border
        float v0, v1, v2, v3;
        if (tx) {  // separable: the four corner rows share the x term, pairs of rows the y and z terms
          const float2 X = __ldg(tx + i), Y0 = __ldg(ty + j), Y1 = __ldg(ty + j + 1), Z0 = __ldg(tz + k),
                       Z1 = __ldg(tz + k + 1);
          v0 = combine_terms(surf, X, Y0, Z0);
          v1 = combine_terms(surf, X, Y1, Z0);
          v2 = combine_terms(surf, X, Y0, Z1);
          v3 = combine_terms(surf, X, Y1, Z1);
        } else {
          v0 = generated_at(P, g.gd, i, j, k);
          v1 = generated_at(P, g.gd, i, j + 1, k);
          v2 = generated_at(P, g.gd, i, j, k + 1);
          v3 = generated_at(P, g.gd, i, j + 1, k + 1);
        }
        b0 = v0 >= iso;
        b1 = v1 >= iso;
        b2 = v2 >= iso;
        b3 = v3 >= iso;
        o[0] = v0;
        if (lj) o[sy] = v1;
        if (lk) o[sz] = v2;
        if (lj && lk) o[szy] = v3;
        if (own_next) {
          float w0, w1, w2, w3;
          if (tx) {
            const float2 X = __ldg(tx + i + 1), Y0 = __ldg(ty + j), Y1 = __ldg(ty + j + 1), Z0 = __ldg(tz + k),
                         Z1 = __ldg(tz + k + 1);
            w0 = combine_terms(surf, X, Y0, Z0);
            w1 = combine_terms(surf, X, Y1, Z0);
            w2 = combine_terms(surf, X, Y0, Z1);
            w3 = combine_terms(surf, X, Y1, Z1);
          } else {
            w0 = generated_at(P, g.gd, i + 1, j, k);
            w1 = generated_at(P, g.gd, i + 1, j + 1, k);
            w2 = generated_at(P, g.gd, i + 1, j, k + 1);
            w3 = generated_at(P, g.gd, i + 1, j + 1, k + 1);
          }
          nx_bits = (unsigned)(w0 >= iso) << 1 | (unsigned)(w1 >= iso) << 3 | (unsigned)(w2 >= iso) << 5 |
                    (unsigned)(w3 >= iso) << 7;
          if (i == cx - 1) {  // the row's last cell also writes the row's last points
            o[1] = w0;
            if (lj) o[sy + 1] = w1;
            if (lk) o[sz + 1] = w2;
            if (lj && lk) o[szy + 1] = w3;
          }
        }
      }
    } else {
      if (valid) {
        b0 = __ldg(p) >= iso;
        b1 = __ldg(p + sy) >= iso;
        b2 = __ldg(p + sz) >= iso;
        b3 = __ldg(p + szy) >= iso;
      }
      if (own_next) {
        nx_bits = (unsigned)(__ldg(p + 1) >= iso) << 1 | (unsigned)(__ldg(p + sy + 1) >= iso) << 3 |
                  (unsigned)(__ldg(p + sz + 1) >= iso) << 5 | (unsigned)(__ldg(p + szy + 1) >= iso) << 7;
      }
    }
    const unsigned m0 = __ballot_sync(0xffffffffu, b0), m1 = __ballot_sync(0xffffffffu, b1),
                   m2 = __ballot_sync(0xffffffffu, b2), m3 = __ballot_sync(0xffffffffu, b3);
    unsigned cs = ((m0 >> lane) & 3u) | ((m1 >> lane) & 3u) << 2 | ((m2 >> lane) & 3u) << 4 | ((m3 >> lane) & 3u) << 6;
    if (own_next) cs = (cs & 0x55u) | nx_bits;
    if (!valid) cs = 0;
    case_of[s * kScanThreads + threadIdx.x] = (uint8_t)cs;
    actbits |= (unsigned)(cs - 1u < 254u) << s;
  }
  return actbits;
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
