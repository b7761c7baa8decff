// Device-side building blocks shared by the DMC and TMC kernels: the grid view, packed cell
// topology, MC polygons (contours) and small helpers.
//
// Arithmetic note: this library is compiled with -fmad=false, so every float/double expression
// written here rounds each operation exactly as the reference's CPU code does when compiled
// without floating-point contraction.  Hot loops that want fused multiply-adds use explicit
// __fmaf_rn / __fma_rn.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ffloat.cuh"
#include "mc_tables.h"

namespace tmc {

// ------------------------------------------------------------------------------------------
// grid view
// ------------------------------------------------------------------------------------------
// Division of a 32-bit unsigned integer by an invariant divisor d >= 1 with one multiply-high, an
// add and two shifts, exact for every 32-bit dividend: the unsigned method with the correction term
// of Granlund & Montgomery, "Division by Invariant Integers using Multiplication" (PLDI 1994, sec. 4):
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, t = mulhi(m, n), q = (t + ((n - t) >> 1)) >> (l - 1)
// (shifts 0 / 0 for d = 1).  Every cell kernel splits cell indices into (i, j, k) with two of these.
struct Div32 {
  uint32_t m = 1, s1 = 0, s2 = 0;  // d = 1
  __host__ void init(uint32_t d) {
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < d) l++;
    m = (uint32_t)((((1ull << l) - d) << 32) / d + 1);
    s1 = l < 1 ? l : 1;
    s2 = l > 1 ? l - 1 : 0;
  }
  __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(m, n);
#else
    const uint32_t t = (uint32_t)(((uint64_t)m * n) >> 32);
#endif
    return (t + ((n - t) >> s1)) >> s2;
  }
};

struct GenParams;  // generators.cuh

struct Grid {
  const float* f;
  int nx, ny, nz;     // points
  double ox, oy, oz;  // origin
  double dx, dy, dz;  // spacing
  double iso;
  float iso_up;       // smallest float >= iso:  (double)f >= iso  <=>  f >= iso_up
  int flags;          // kGridFlip | kGridNormal64 | kGridPos64
  int64_t vbase;      // index of cell 0 in the launch's cell space (0 for a single volume)
  double inv2[3];     // 1 / (2 * spacing), for the central-difference gradients
  float inv2f[3];     // the same rounded to float
  // float forms for the float32 paths, made once on the host (a float64 conversion per vertex runs
  // on the float64 pipe): origin and spacing as float pairs (hi + lo within 2^-48 relative of the
  // double), the isovalue rounded to float
  float org_hi[3], org_lo[3], sp_hi[3], sp_lo[3];
  float inv2_hi[3], inv2_lo[3];  // 1 / (2 * spacing)
  float iso_f;
  Div32 div_cx, div_cy;  // division by nx - 1 and ny - 1 (cell index -> i, j, k); set_divisors()
  // fused generation (single-volume launches): the classification evaluates the field from `gen` at
  // the float32 spacing gd instead of reading f, and writes each point once to gen_out (== f), which
  // the later passes read
  const GenParams* gen;
  float* gen_out;
  float gd[3];
  __host__ void set_divisors() {
    div_cx.init((uint32_t)(nx - 1));
    div_cy.init((uint32_t)(ny - 1));
  }
  __host__ __device__ int cx() const { return nx - 1; }
  __host__ __device__ int cy() const { return ny - 1; }
  __host__ __device__ int cz() const { return nz - 1; }
  __host__ __device__ int64_t ncells() const { return (int64_t)(nx - 1) * (ny - 1) * (nz - 1); }
  __device__ __forceinline__ float at(int i, int j, int k) const {
    return __ldg(f + ((int64_t)k * ny + j) * nx + i);
  }
  __host__ __device__ __forceinline__ int64_t cell_index(int i, int j, int k) const {
    return ((int64_t)k * (ny - 1) + j) * (nx - 1) + i;
  }
  // index of cell (i, j, k) in the launch's cell space (per-cell scratch arrays)
  __host__ __device__ __forceinline__ int64_t vcell(int i, int j, int k) const { return vbase + cell_index(i, j, k); }
};

// Grid::flags: per-volume output choices (a batch mixes requests with different flags)
constexpr int kGridFlip = 1;      // DMC normals from the negated gradient
constexpr int kGridNormal64 = 2;  // DMC: float64 normals (kept while the mesh is simplified)
constexpr int kGridPos64 = 4;     // TMC: float64 edge-vertex positions and normals

// The cells one launch works on: a single volume, or a batch of volumes laid out one after another
// in a linear cell space.  In a batch every volume starts on a scan-tile boundary (kScanTile cells),
// so a tile never straddles two volumes; the rest of a volume's last tile is padding whose records
// stay empty.  Per-cell scratch (records, offsets) is indexed in this space.
struct CellSpace {
  Grid one;                 // single-volume launches
  const Grid* grids;        // batch: grid of each volume (vbase set), else nullptr
  const int32_t* tile_vol;  // batch: volume of each tile
  int64_t n;                // cells in the space, padding included
  __device__ __forceinline__ Grid grid_of_tile(int64_t tile) const {
    if (!grids) return one;
    return grids[__ldg(tile_vol + tile)];
  }
};

// Listed cells.  The classification lists, per scan tile, the cells whose MC case is neither 0 nor
// 255 (12 % of the cells of the 512^3 dense-ambiguity field, 3 % of a smooth one); every per-cell
// array after it (records, in-tile cell offsets, vertex and face offsets) holds only those, in cell
// order, at slot = tile * kScanTile + rank in the tile, so the passes read and write 4 to 16 bytes
// per listed cell instead of per cell.  CellMask, one per 32 cells, says which cells are listed and
// how many listed cells of the tile come before the word; a cell's slot is one 8-byte load and a
// population count away.
struct CellMask {
  uint32_t bits;  // listed cells among the word's 32
  uint32_t pre;   // listed cells of the tile before the word
};
constexpr int kTileShift = 11;  // kScanTile = 2048 cells per scan tile
__device__ __forceinline__ uint32_t listed_slot(const CellMask* mask, uint32_t vc) {
  const uint2 a = __ldg(reinterpret_cast<const uint2*>(mask) + (vc >> 5));
  return ((vc >> kTileShift) << kTileShift) + a.y + __popc(a.x & ((1u << (vc & 31)) - 1u));
}
// number of listed cells of a tile
__device__ __forceinline__ uint32_t tile_listed(const CellMask* mask, int64_t tile) {
  const uint2 a = __ldg(reinterpret_cast<const uint2*>(mask) + (tile << (kTileShift - 5)) + 63);
  return a.y + __popc(a.x);
}
// Chunk q of 32 slots for the kernels that walk the listed cells.  Every tile's listed cells sit in
// its front slots, so the chunks run over the tiles first (chunk r of a run covers slots
// 32 * (r / W) .. + 31 of the run's tile r % W): consecutive warps take the front slots of
// consecutive tiles.  Numbered tile by tile instead, the warps whose index is a multiple of 64 apart
// would take the same part of every tile and a few of them would get all the work.  The runs are
// windows of kChunkWindow consecutive tiles (a few z-planes of a volume), taken in order, so that the
// cells processed at any moment, and the field around them, stay within a narrow band that the L2
// holds.
constexpr int64_t kChunkWindow = 512;
__host__ __device__ __forceinline__ void slot_chunk(int64_t q, int64_t tiles, int64_t& tile, uint32_t& first) {
  const int64_t per = kChunkWindow << (kTileShift - 5);  // chunks of a full window (32 slots each)
  const int64_t win = q / per;
  const int64_t t0 = win * kChunkWindow;
  const int64_t w = tiles - t0 < kChunkWindow ? tiles - t0 : kChunkWindow;  // tiles in this window
  const int64_t r = q - win * per;
  const int64_t part = r / w;
  tile = t0 + (r - part * w);
  first = (uint32_t)(tile << kTileShift) + (uint32_t)part * 32u;
}
// the cell behind a slot (cell: in-tile cell offsets of the listed cells)
__device__ __forceinline__ uint32_t slot_cell(const uint16_t* cell, uint32_t slot) {
  return ((slot >> kTileShift) << kTileShift) + __ldg(cell + slot);
}

inline CellSpace single_space(const Grid& g) {
  CellSpace cs;
  cs.one = g;
  cs.one.vbase = 0;
  cs.grids = nullptr;
  cs.tile_vol = nullptr;
  cs.n = g.ncells();
  return cs;
}

// ------------------------------------------------------------------------------------------
// packed topology lookups (4 bits per entry)
// ------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ int nib(uint64_t w, int i) { return (int)((w >> (4 * i)) & 0xF); }
__host__ __device__ __forceinline__ int edge_v0(int e) { return nib(TMC_PK_EDGE_V0, e); }
__host__ __device__ __forceinline__ int edge_v1(int e) { return nib(TMC_PK_EDGE_V1, e); }
__host__ __device__ __forceinline__ int edge_off(int e) { return nib(TMC_PK_EDGE_OFF, e); }   // di|dj<<1|dk<<2
__host__ __device__ __forceinline__ int edge_axis(int e) { return nib(TMC_PK_EDGE_AXIS, e); }
__host__ __device__ __forceinline__ int quad_slot(int e, int neg) {
  return neg ? nib(TMC_PK_QUAD_SLOT1, e) : nib(TMC_PK_QUAD_SLOT0, e);
}
__host__ __device__ __forceinline__ uint32_t face_v_pack(int f) {
  constexpr uint32_t P[6] = {TMC_PK_FACE_V0, TMC_PK_FACE_V1, TMC_PK_FACE_V2,
                             TMC_PK_FACE_V3, TMC_PK_FACE_V4, TMC_PK_FACE_V5};
  return P[f];
}
__host__ __device__ __forceinline__ uint32_t face_e_pack(int f) {
  constexpr uint32_t P[6] = {TMC_PK_FACE_E0, TMC_PK_FACE_E1, TMC_PK_FACE_E2,
                             TMC_PK_FACE_E3, TMC_PK_FACE_E4, TMC_PK_FACE_E5};
  return P[f];
}
// single segment of the face cases that need no decider: face-local edge a -> edge b
#define TMC_PK_FACE_RULE_A 0x303220210031100ull
#define TMC_PK_FACE_RULE_B 0x11300120223030ull

__host__ __device__ __forceinline__ bool case_ambiguous(unsigned c) {
  const uint64_t w = (c < 128) ? ((c < 64) ? TMC_AMBIGUOUS_W0 : TMC_AMBIGUOUS_W1)
                               : ((c < 192) ? TMC_AMBIGUOUS_W2 : TMC_AMBIGUOUS_W3);
  return (w >> (c & 63)) & 1ull;
}
// edges crossed by the isosurface for case c (bit e)
__host__ __device__ __forceinline__ uint32_t case_edge_mask(unsigned c) {
  uint32_t m = 0;
#pragma unroll
  for (int e = 0; e < 12; e++) m |= (((c >> edge_v0(e)) ^ (c >> edge_v1(e))) & 1u) << e;
  return m;
}

// ------------------------------------------------------------------------------------------
// contours of the MC polygon, packed in 64 bits:
//   nibbles 0..11  the edges of all contours in order (contour t starts after contours 0..t-1)
//   nibbles 12..15 the size of contour 0..3 (0 = no contour)
// ------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ int cnt_size(uint64_t c, int t) { return nib(c, 12 + t); }
__host__ __device__ __forceinline__ int cnt_count(uint64_t c) {
  return (cnt_size(c, 0) > 0) + (cnt_size(c, 1) > 0) + (cnt_size(c, 2) > 0) + (cnt_size(c, 3) > 0);
}
__host__ __device__ __forceinline__ int cnt_start(uint64_t c, int t) {
  int s = 0;
  for (int q = 0; q < t; q++) s += cnt_size(c, q);
  return s;
}
__host__ __device__ __forceinline__ int cnt_edge(uint64_t c, int flat) { return nib(c, flat); }

__host__ __device__ __forceinline__ int ctz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

// Connect oriented segments into closed contours, each starting at its lowest edge -- the
// connect loop of mc_polygon (cpp_dmc/DualMarchingCubes.cpp:443-463) and p_slice
// (mc/MarchingCubes.cpp:690-709).  `to` holds the next edge of every crossed edge (nibble e),
// `emask` the crossed edges.
__host__ __device__ __forceinline__ uint64_t connect_contours(uint64_t to, uint32_t emask) {
  uint64_t out = 0;
  int flat = 0, t = 0;
  uint32_t rem = emask;
  while (rem && t < 4) {
    const int start = ctz32(rem);
    int e = start, sz = 0;
    do {
      out |= (uint64_t)e << (4 * flat);
      flat++;
      sz++;
      rem &= ~(1u << e);
      e = nib(to, e);
    } while (e != start && sz < 12);
    out |= (uint64_t)sz << (4 * (12 + t));
    t++;
  }
  return out;
}

// Oriented segments of one face: fc = face case (bit b: face vertex b >= iso), sep = the decider
// branch for the two ambiguous face cases (6, 9).  Follows the face-case switch of
// cpp_dmc/DualMarchingCubes.cpp:357-425 / mc/MarchingCubes.cpp:495-668.
__host__ __device__ __forceinline__ void face_segments(int fc, int sep, uint32_t fe, uint64_t& to) {
  auto set = [&](int a, int b) {
    const int ea = nib(fe, a), eb = nib(fe, b);
    to = (to & ~(0xFull << (4 * ea))) | ((uint64_t)eb << (4 * ea));
  };
  if (fc == 6) {
    if (sep) { set(3, 0); set(1, 2); }
    else { set(1, 0); set(3, 2); }
  } else if (fc == 9) {
    if (sep) { set(0, 1); set(2, 3); }
    else { set(0, 3); set(2, 1); }
  } else if (fc != 0 && fc != 15) {
    set(nib(TMC_PK_FACE_RULE_A, fc), nib(TMC_PK_FACE_RULE_B, fc));
  }
}

__host__ __device__ __forceinline__ int face_case(unsigned cs, uint32_t fv) {
  return (int)(((cs >> nib(fv, 0)) & 1) | ((cs >> nib(fv, 1)) & 1) << 1 | ((cs >> nib(fv, 2)) & 1) << 2 |
               ((cs >> nib(fv, 3)) & 1) << 3);
}

// asymptotic decider, float64 (cpp_dmc/DualMarchingCubes.h:330)
__host__ __device__ __forceinline__ double decider(double f0, double f1, double f2, double f3) {
  return (f0 * f3 - f1 * f2) / (f0 + f3 - f1 - f2);
}

// Contour of an unambiguous case from the packed table (size nibble, then edges).
__host__ __device__ __forceinline__ uint64_t table_contour(uint64_t w) {
  const int sz = (int)(w & 0xF);
  return (w >> 4) | ((uint64_t)sz << 48);
}

// decider(f0..f3) >= iso, decided in float-float when the margin is clear, else in float64.
// The reference evaluates (f0*f3 - f1*f2) / (f0 + f3 - f1 - f2) in double: the products are exact,
// the difference and the sum round once or twice; both are reproduced within ~2^-46.
// Out of line: ambiguous faces are rare and six inlined copies would bloat every caller.
inline __host__ __device__ __noinline__ bool decider_ge(float f0, float f1, float f2, float f3, double iso,
                                                 ffx::ff iso_ff) {
  using namespace ffx;
  const ff a = two_prod(f0, f3), b = two_prod(f1, f2);
  const ff num = ff_sub(a, b);
  const ff den = ff_sub(ff_sub(ff_add(ff_from(f0), ff_from(f3)), ff_from(f1)), ff_from(f2));
  if (den.hi != 0.0f) {
    const ff q = ff_div(num, den);
    const ff d = ff_sub(q, iso_ff);
    const float mag = fabsf(a.hi) + fabsf(b.hi);
    const float err = mag * 0x1p-44f / fabsf(den.hi) + fabsf(q.hi) * 0x1p-44f + fabsf(iso_ff.hi) * 0x1p-46f +
                      (fabsf(f0) + fabsf(f1) + fabsf(f2) + fabsf(f3)) * 0x1p-44f * fabsf(q.hi) / fabsf(den.hi);
    if (d.hi > err) return true;
    if (d.hi < -err) return false;
  }
  return decider(f0, f1, f2, f3) >= iso;
}

// DMC MC polygon (mc_polygon, cpp_dmc/DualMarchingCubes.cpp:328-487): table contour for the
// unambiguous cases, face rules with the decider (>= iso) for the ambiguous ones.
__device__ __forceinline__ uint64_t dmc_polygon(unsigned cs, const float u[8], double iso, const uint64_t* case_contour) {
  if (!case_ambiguous(cs)) return table_contour(case_contour[cs]);
  const ffx::ff iso_ff = ffx::ff_from_double(iso);
  uint64_t to = ~0ull;
#pragma unroll
  for (int f = 0; f < 6; f++) {
    const uint32_t fv = face_v_pack(f);
    const int fc = face_case(cs, fv);
    int sep = 0;
    if (fc == 6 || fc == 9) sep = decider_ge(u[nib(fv, 0)], u[nib(fv, 1)], u[nib(fv, 2)], u[nib(fv, 3)], iso, iso_ff);
    face_segments(fc, sep, face_e_pack(f), to);
  }
  return connect_contours(to, case_edge_mask(cs));
}

// ------------------------------------------------------------------------------------------
// misc
// ------------------------------------------------------------------------------------------
struct DevFlags {
  unsigned int overflow;   // a capacity check failed
  unsigned int numeric;    // NaN / Inf seen
  unsigned int timeout;    // a bounded wait gave up
  unsigned int pad;
  unsigned long long counters[8];
};

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Launch shapes of a context.  Every setting gives identical meshes; they trade the latency of a
// small call against the throughput of a large one.  Defaults follow the SM count; tmc_ctx_autotune
// measures candidates on the caller's own volumes.
struct Tuning {
  int sms = 1;
  int64_t group_lanes = 0;        // lanes the projection pass may fill with lane groups (0: one thread per vertex)
  int64_t warp_list_max = 0;      // float64 fallback lists up to this length run one warp per vertex
  int vertex_blocks_per_sm = 32;  // grid cap of the per-vertex passes (rounded to whole waves)
  int emit_blocks_per_sm = 8;     // grid cap of the TMC emission kernel
  int quad_blocks_per_sm = 1;     // grid of the DMC quad pass (whole waves)
  int64_t slab_bytes = (int64_t)32 << 20;  // host-field slab depth
  int max_slabs = 16;             // host-field slabs per field
  static Tuning defaults(int sms) {
    Tuning t;
    t.sms = sms;
    t.group_lanes = (int64_t)sms * 24 * 32;
    t.warp_list_max = (int64_t)sms * 32;
    return t;
  }
};

// Blocks of `kernel` that fit on one SM at `threads` threads per block (the occupancy calculator;
// registers and shared memory decide).
template <typename K>
inline int resident_blocks(K kernel, int threads) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, 0) != cudaSuccess || b < 1) b = 1;
  return b;
}

// Grid of a grid-stride launch: a whole number of waves (resident blocks per SM x SMs), the one
// nearest to `per_sm` blocks per SM, and no more blocks than `threads`-item groups.  A grid of
// 1.3 waves would run its last 0.3 wave alone, as long as a full one.
inline int64_t wave_grid(int resident, int sms, int64_t per_sm, int64_t items, int threads) {
  const int64_t waves = per_sm <= resident ? 1 : (per_sm + resident / 2) / resident;
  const int64_t g = waves * resident * (int64_t)sms;
  const int64_t need = (items + threads - 1) / threads;
  return need < 1 ? 1 : (need < g ? need : g);
}

// Classification may start before the whole field is on the device (a host field copied in z
// slabs): the scan tiles below tile_end may run once `ready` has completed.  Gates come in order,
// the last one covers every tile.
struct TileGate {
  int64_t tile_end;
  cudaEvent_t ready;
};

}  // namespace tmc
