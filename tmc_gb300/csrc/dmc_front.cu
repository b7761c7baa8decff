// Dual Marching Cubes front end: per-cell classification, MC polygons, vertex representatives
// and quads, emitted in the reference's order without hash tables.
//
// Order.  The reference CPU path (cpp_dmc/DualMarchingCubes.cpp:16-50, :97-192) appends one
// vertex per contour in cell order, stores quads in a std::map keyed by the dual grid edge
// (3*global_index + axis) and walks the map in key order (DualMarchingCubes.h:663); vertices that
// no complete quad uses are then dropped (DualMarchingCubes.h:685).  A contour's vertex is used
// exactly when one of its edges is an interior grid edge (all four cells around it exist), and a
// quad exists exactly for every crossed interior edge.  So:
//   vertex index = #used contours in earlier cells + rank of the contour among the cell's used ones
//   quad index   = #crossed interior edges owned by earlier grid points + rank of the axis
// Both are exclusive prefix sums over cells; no atomics, no hash table, deterministic output.
//
// Kernels:
//   dmc_classify_kernel  case, contours, per-cell record (counts + edge->vertex rank map) and
//                        per-tile sums for the scan
//   dmc_offsets_kernel   in-tile scan -> per-cell vertex / quad offsets
//   dmc_vertex_setup_kernel, dmc_project_kernel (dmc_project_group_kernel for small meshes),
//   dmc_vertex_finish_kernel
//                        vertex representatives (cpp_dmc representative/projection) in float32
//                        and float-float, normals, positions
//   dmc_vertex_kernel    the vertices those leave, with every float64 fallback
//   dmc_vertex_warp_kernel  the reference's 26x26 retry (and short lists whole), one warp per vertex
//   dmc_quad_kernel      each cell emits the quads of its crossed interior edges 0, 3, 8 by
//                        looking up the four cells around the edge
#include <cstdio>

#include "common.cuh"
#include "dmc.h"
#include "dmc_cell.cuh"
#include "dmc_repr.cuh"
#include "scan.cuh"

namespace tmc {

static_assert(sizeof(repr::ProjRecord) == kProjRecordBytes, "record size");

__constant__ uint64_t c_case_contour[256] = TMC_CASE_CONTOUR_INIT;

// ------------------------------------------------------------------------------------------
// classification (per-cell helpers in dmc_cell.cuh)
// ------------------------------------------------------------------------------------------
// One block per kScanTile consecutive cells (linear order).  Pass 1: every cell's MC case from the
// warp-ballot corner rows (tile_cases: one coalesced load per corner row and warp, no per-cell
// gather); the cells with a case other than 0 and 255 are listed in cell order (list_tile).  Pass 2:
// the contours and records of the listed cells with an unambiguous case, written densely at their
// slots with their in-tile offsets, and the tile's packed (vertices << 32 | quads) sum.  Listed cells
// with an ambiguous case (the asymptotic decider, ~1 % of the cells) go by slot to amb_list for
// dmc_amb_kernel, which runs them densely instead of stalling every warp here on a few lanes.
template <bool kGen>
__global__ void __launch_bounds__(kScanThreads, 6) dmc_classify_kernel(CellSpace space, int64_t tile0, uint32_t* rec,
                                                                   uint16_t* cellof, uint8_t* ccase, CellMask* mask,
                                                                   unsigned long long* tile_sums,
                                                                   unsigned long long* stats, uint32_t* amb_list,
                                                                   unsigned* amb_n) {
  const int64_t tile = tile0 + blockIdx.x;
  __shared__ uint64_t cc[256];
  __shared__ uint16_t act_list[kScanTile];
  __shared__ uint8_t case_of[kScanTile];
  __shared__ uint32_t wmask[kScanTile / 32], wpre[kScanTile / 32];
  __shared__ int total;
  __shared__ unsigned long long tile_sum;
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  if (threadIdx.x == 0) tile_sum = 0;
  const Grid g = space.grid_of_tile(tile);
  const int64_t vbase = tile * kScanTile;  // first cell of the tile in the space
  const int lane = threadIdx.x & 31;
  const unsigned actbits = tile_cases<kGen>(g, space.n, vbase, case_of);
  const int na = list_tile(actbits, tile, mask, wmask, wpre, act_list, &total);
  // pass 2: records of the listed cells
  unsigned long long local = 0, amb = 0, nact = 0;
  for (int a = threadIdx.x; a < na; a += blockDim.x) {
    const int off = act_list[a];
    const uint32_t slot = (uint32_t)(vbase + a);
    const unsigned cs = case_of[off];
    const bool ambiguous = case_ambiguous(cs);
    cellof[slot] = (uint16_t)off;
    ccase[slot] = (uint8_t)cs;
    if (!ambiguous) {
      int i, j, k;
      cell_ijk(g, vbase + off - g.vbase, i, j, k);
      const uint32_t r = record_from_contours(g, i, j, k, cs, table_contour(cc[cs]), false);
      rec[slot] = r;
      local += ((unsigned long long)rec_nv(r) << 32) | (unsigned long long)rec_nq(r);
      nact += r != 0;
    }
    amb += ambiguous;
    const unsigned am = __activemask();
    const unsigned bal = __ballot_sync(am, ambiguous);
    if (bal) {
      const int leader = __ffs(bal) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(amb_n, (unsigned)__popc(bal));
      base = __shfl_sync(am, base, leader);
      if (ambiguous) amb_list[base + __popc(bal & ((1u << lane) - 1u))] = slot;
    }
  }
  for (int o = 16; o; o >>= 1) {
    local += __shfl_down_sync(0xffffffffu, local, o);
    amb += __shfl_down_sync(0xffffffffu, amb, o);
    nact += __shfl_down_sync(0xffffffffu, nact, o);
  }
  if (lane == 0 && local) atomicAdd(&tile_sum, local);
  // stats[0]: cells with a record (a used contour, an owned quad or the ambiguous flag); the
  // ambiguous cells' records are never empty, so they count here too
  if (lane == 0 && amb) atomicAdd(stats + 1, amb);
  if (lane == 0 && (nact | amb)) atomicAdd(stats + 0, nact + amb);
  __syncthreads();
  if (threadIdx.x == 0) tile_sums[tile] = tile_sum;
}

// The ambiguous listed cells: MC polygon with the asymptotic decider (float-float, float64 near the
// isovalue), record, and their counts added to their tile's sum (after the classification wrote it).
__global__ void __launch_bounds__(128) dmc_amb_kernel(CellSpace space, const uint16_t* cellof, uint32_t* rec,
                                                      unsigned long long* tile_sums, const uint32_t* list,
                                                      const unsigned* count) {
  __shared__ uint64_t cc[256];
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  const unsigned na = *count;
  for (unsigned a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) {
    const uint32_t slot = list[a];
    const int64_t tile = slot >> kTileShift;
    const Grid g = space.grid_of_tile(tile);
    int i, j, k;
    cell_ijk(g, slot_cell(cellof, slot) - g.vbase, i, j, k);
    float u[8];
    load_corners(g, i, j, k, u);
    const uint32_t r = classify_active(g, i, j, k, mc_case(u, g.iso_up), u, cc);
    rec[slot] = r;
    const unsigned long long add = ((unsigned long long)rec_nv(r) << 32) | (unsigned long long)rec_nq(r);
    if (add) atomicAdd(tile_sums + tile, add);
  }
}

// In-tile exclusive scan of the listed cells' records -> their vertex and quad offsets (blocked:
// 16-byte record loads and offset stores over the tile's slots, one block scan of the thread
// totals), and two entries per vertex: the slot of the cell that generates it and its rank there.
__global__ void __launch_bounds__(32 * kOffsetWarps) dmc_offsets_kernel(const CellMask* mask, const uint32_t* rec,
                                                                       const unsigned long long* tile_off,
                                                                       int64_t tiles, int32_t* voff, int32_t* qoff,
                                                                       uint32_t* vwork, uint8_t* vrank) {
  const int lane = threadIdx.x & 31;
  const int64_t tile = (int64_t)blockIdx.x * kOffsetWarps + (threadIdx.x >> 5);
  if (tile >= tiles) return;  // the whole warp
  const int64_t base = tile * kScanTile;
  const int64_t end = base + tile_listed(mask, tile);
  unsigned long long carry = tile_off[tile];
  for (int64_t step = base; step < end; step += kOffsetStep) {  // warp-uniform
    const int64_t first = step + (int64_t)lane * kScanItems;
    uint32_t r[kScanItems];
    load8(rec, first, end, r);
    unsigned long long sum = 0;
#pragma unroll
    for (int s = 0; s < kScanItems; s++) sum += ((unsigned long long)rec_nv(r[s]) << 32) | rec_nq(r[s]);
    const unsigned long long inc = warp_inclusive_scan(sum);
    unsigned long long pre = carry + inc - sum;
    carry += __shfl_sync(0xffffffffu, inc, 31);
    int32_t vo[kScanItems], qo[kScanItems];
#pragma unroll
    for (int s = 0; s < kScanItems; s++) {
      vo[s] = (int32_t)(pre >> 32);
      qo[s] = (int32_t)(pre & 0xffffffffull);
      pre += ((unsigned long long)rec_nv(r[s]) << 32) | rec_nq(r[s]);
    }
    store8(voff, first, end, vo);
    store8(qoff, first, end, qo);
#pragma unroll
    for (int s = 0; s < kScanItems; s++)
      for (int q = 0; q < rec_nv(r[s]); q++) {  // empty beyond the listed cells
        vwork[vo[s] + q] = (uint32_t)(first + s);
        vrank[vo[s] + q] = (uint8_t)q;
      }
  }
}

// ------------------------------------------------------------------------------------------
// vertices: one thread per output vertex (work list from the offsets kernel).  The representative
// comes from representative_fast (dmc_repr.cuh): float32 search with certified float-float
// rounding, bit-identical to the reference's float/double arithmetic.
// ------------------------------------------------------------------------------------------
// estimateGradient at a grid point (cpp_dmc/UniformGrid.cpp:512-540): central differences with
// the reference's border indexing ((i<0) ? 0 : (i>=max) ? max-i : i).
__device__ __forceinline__ int grad_index(int i, int max) { return (i < 0) ? 0 : (i >= max) ? max - i : i; }
// Central differences at a grid point, exact as float pairs (the reference's float64 difference
// of two floats); the 1/(2*spacing) factor is applied after the interpolation.
__device__ __forceinline__ void point_diff_ff(const Grid& g, int i, int j, int k, ffx::ff out[3]) {
  const int i0 = grad_index(i - 1, g.nx), i1 = grad_index(i + 1, g.nx);
  const int j0 = grad_index(j - 1, g.ny), j1 = grad_index(j + 1, g.ny);
  const int k0 = grad_index(k - 1, g.nz), k1 = grad_index(k + 1, g.nz);
  out[0] = ffx::two_sum(g.at(i1, j, k), -g.at(i0, j, k));
  out[1] = ffx::two_sum(g.at(i, j1, k), -g.at(i, j0, k));
  out[2] = ffx::two_sum(g.at(i, j, k1), -g.at(i, j, k0));
}
// a + t*(b - a) in float-float
__device__ __forceinline__ ffx::ff ff_lerp(ffx::ff a, ffx::ff b, float t) {
  return ffx::ff_add(a, ffx::ff_mul_f(ffx::ff_sub(b, a), t));
}

struct Normal64 {
  double n[3];
};
// The reference's float64 normal (UniformGrid::normal on estimateGradient values), for the rare
// vertices whose gradients cancel so much that the float-float result would lose its margin.
__device__ __noinline__ Normal64 normal_f64(const Grid g, int i, int j, int k, double pu, double pv, double pw,
                                            int flip) {
  const double inv2d[3] = {1.0 / (2 * g.dx), 1.0 / (2 * g.dy), 1.0 / (2 * g.dz)};
  double G[8][3];
  for (int q = 0; q < 8; q++) {
    const int a = i + (q & 1), b = j + ((q >> 1) & 1), c = k + ((q >> 2) & 1);
    const int i0 = grad_index(a - 1, g.nx), i1 = grad_index(a + 1, g.nx);
    const int j0 = grad_index(b - 1, g.ny), j1 = grad_index(b + 1, g.ny);
    const int k0 = grad_index(c - 1, g.nz), k1 = grad_index(c + 1, g.nz);
    G[q][0] = ((double)g.at(i1, b, c) - (double)g.at(i0, b, c)) * inv2d[0];
    G[q][1] = ((double)g.at(a, j1, c) - (double)g.at(a, j0, c)) * inv2d[1];
    G[q][2] = ((double)g.at(a, b, k1) - (double)g.at(a, b, k0)) * inv2d[2];
  }
  const double uu = pu, vv = pv, ww = pw;
  double nv3[3];
  for (int d = 0; d < 3; d++) {
    double gq[8];
    for (int q = 0; q < 8; q++) gq[q] = flip ? G[q][d] * -1. : G[q][d];
    nv3[d] = (1 - ww) * ((1 - vv) * ((1 - uu) * gq[0] + uu * gq[1]) + vv * ((1 - uu) * gq[2] + uu * gq[3])) +
             ww * ((1 - vv) * ((1 - uu) * gq[4] + uu * gq[5]) + vv * ((1 - uu) * gq[6] + uu * gq[7]));
  }
  const double s = sqrt(nv3[0] * nv3[0] + nv3[1] * nv3[1] + nv3[2] * nv3[2]);
  Normal64 r;
  for (int d = 0; d < 3; d++) r.n[d] = nv3[d] / s;
  return r;
}
__device__ __forceinline__ void point_gradient_f(const Grid& g, int i, int j, int k, float inv2d[3], float out[3]) {
  const int i0 = grad_index(i - 1, g.nx), i1 = grad_index(i + 1, g.nx);
  const int j0 = grad_index(j - 1, g.ny), j1 = grad_index(j + 1, g.ny);
  const int k0 = grad_index(k - 1, g.nz), k1 = grad_index(k + 1, g.nz);
  out[0] = (g.at(i1, j, k) - g.at(i0, j, k)) * inv2d[0];
  out[1] = (g.at(i, j1, k) - g.at(i, j0, k)) * inv2d[1];
  out[2] = (g.at(i, j, k1) - g.at(i, j, k0)) * inv2d[2];
}

constexpr int kVertexThreads = 128;

// The current volume's grid and the constants derived from it, cached per thread (a batch mixes
// volumes; consecutive vertices mostly share one).
struct GridCache {
  int vol = -1;
  Grid g{};
  ffx::ff iso_ff{0, 0};
  float inv2d[3] = {0, 0, 0};
  ffx::ff inv2d_ff[3] = {{0, 0}, {0, 0}, {0, 0}};
  __device__ __forceinline__ void load(const CellSpace& space, uint32_t vcell) {
    const int v = space.grids ? __ldg(space.tile_vol + vcell / kScanTile) : 0;
    if (v == vol) return;
    vol = v;
    g = space.grids ? space.grids[v] : space.one;
    iso_ff = ffx::ff_from_double(g.iso);
    for (int d = 0; d < 3; d++) {
      inv2d[d] = (float)g.inv2[d];
      inv2d_ff[d] = ffx::ff_from_double(g.inv2[d]);
    }
  }
};

// The contour behind vertex `rank` of a cell: corners, MC polygon, and the edge points and bounding
// boxes of all its contours (slice, cpp_dmc/DualMarchingCubes.cpp:114-136).
struct VertexContour {
  float u[8];
  uint64_t c;
  repr::Boxes bx;
  float pts[36];
  int tsel, tstart;
};
__device__ __forceinline__ bool vertex_contour(const Grid& g, int i, int j, int k, int rank, const uint64_t* cc,
                                               ffx::ff iso_ff, VertexContour& V) {
  load_corners(g, i, j, k, V.u);
  const unsigned cs = mc_case(V.u, g.iso_up);
  V.c = dmc_polygon(cs, V.u, g.iso, cc);
  const int ncnt = cnt_count(V.c);
  int flat = 0, used_seen = 0;
  V.tsel = -1;
  V.tstart = 0;
  for (int t = 0; t < ncnt; t++) {
    V.bx.b[t][0][0] = 1; V.bx.b[t][0][1] = 0;
    V.bx.b[t][1][0] = 1; V.bx.b[t][1][1] = 0;
    V.bx.b[t][2][0] = 1; V.bx.b[t][2][1] = 0;
    const int sz = cnt_size(V.c, t);
    bool used = false;
    for (int q = 0; q < sz; q++) {
      const int e = cnt_edge(V.c, flat + q);
      used = used || edge_interior(g, i, j, k, e);
      bool fb = false;
      const float l = repr::edge_param_fast(e, V.u, g.iso, iso_ff, fb);
      float ui[3];
      repr::local_from_param(e, l, ui);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        V.pts[3 * (flat + q) + d] = ui[d];
        V.bx.b[t][d][0] = V.bx.b[t][d][0] > ui[d] ? ui[d] : V.bx.b[t][d][0];
        V.bx.b[t][d][1] = V.bx.b[t][d][1] < ui[d] ? ui[d] : V.bx.b[t][d][1];
      }
    }
    if (used) {
      if (used_seen == rank) {
        V.tsel = t;
        V.tstart = flat;
      }
      used_seen++;
    }
    flat += sz;
  }
  return V.tsel >= 0;
}

// Position, normal and local coordinates of vertex vidx at local coordinates p of cell (i, j, k).
// p64: the float64 local coordinates when they are not the floats p (the reference's unrounded mean
// point, for contours without any valid projection sample), else null.
// kFF: the float-float normal path (float64 normals kept for the simplification) is compiled in
template <bool kFF = true>
__device__ __forceinline__ void vertex_outputs(const GridCache& G, int i, int j, int k, int64_t cell,
                                               const float p[3], const double* p64, int64_t vidx,
                                               const DmcVertexOut& out, int flip, repr::Stats& st) {
  const Grid& g = G.g;
  const int64_t o = 3 * vidx;
  // a simplified volume: its float32 positions and normals are written after the passes, from the
  // float64 positions and the float-pair normals kept here
  const bool keep64 = out.n64 && (g.flags & kGridNormal64);
  float2* n2 = reinterpret_cast<float2*>(out.n64);
  // position: UniformGrid::position (cpp_dmc/UniformGrid.h:300-305)
  const double lx = p64 ? p64[0] : (double)p[0], ly = p64 ? p64[1] : (double)p[1], lz = p64 ? p64[2] : (double)p[2];
  const double px = g.ox + (i + lx) * g.dx;
  const double py = g.oy + (j + ly) * g.dy;
  const double pz = g.oz + (k + lz) * g.dz;
  if (!keep64) {
    out.v[o] = (float)px;
    out.v[o + 1] = (float)py;
    out.v[o + 2] = (float)pz;
  }
  if (out.v64) {
    out.v64[o] = px;
    out.v64[o + 1] = py;
    out.v64[o + 2] = pz;
  }
  // normal: trilinear interpolation of the 8 corner gradients, normalised (UniformGrid::normal,
  // cpp_dmc/UniformGrid.h:286-298).  When it is kept for the simplification merges it is computed
  // in float-float (relative error ~2^-40, far below the float32 output's 2^-24) on the FP32 pipes.
  if (p64) {
    // float64 local coordinates: the reference's float64 normal at them
    const Normal64 nf = normal_f64(g, i, j, k, lx, ly, lz, flip);
    for (int d = 0; d < 3; d++) {
      if (keep64) {
        const ffx::ff x = ffx::ff_from_double(nf.n[d]);
        n2[o + d] = make_float2(x.hi, x.lo);
      } else {
        out.n[o + d] = (float)nf.n[d];
      }
    }
    st.normal_f64++;
  } else if (kFF && keep64) {
    ffx::ff Gq[8][3];
#pragma unroll
    for (int q = 0; q < 8; q++) point_diff_ff(g, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1), Gq[q]);
    ffx::ff nv3[3];
    float scale = 0;  // largest |difference| * 1/(2 spacing): the size of the interpolation's inputs
#pragma unroll
    for (int d = 0; d < 3; d++) {
      float md = 0;
#pragma unroll
      for (int q = 0; q < 8; q++) md = fmaxf(md, fabsf(Gq[q][d].hi));
      scale = fmaxf(scale, md * G.inv2d[d]);
      const ffx::ff a0 = ff_lerp(Gq[0][d], Gq[1][d], p[0]), a1 = ff_lerp(Gq[2][d], Gq[3][d], p[0]);
      const ffx::ff a2 = ff_lerp(Gq[4][d], Gq[5][d], p[0]), a3 = ff_lerp(Gq[6][d], Gq[7][d], p[0]);
      const ffx::ff b0 = ff_lerp(a0, a1, p[1]), b1 = ff_lerp(a2, a3, p[1]);
      const ffx::ff t = ffx::ff_mul(ff_lerp(b0, b1, p[2]), G.inv2d_ff[d]);
      nv3[d] = flip ? ffx::ff_neg(t) : t;
    }
    const ffx::ff dot =
        ffx::ff_add(ffx::ff_add(ffx::ff_mul(nv3[0], nv3[0]), ffx::ff_mul(nv3[1], nv3[1])), ffx::ff_mul(nv3[2], nv3[2]));
    // 1/sqrt(dot): float estimate and one Newton step in float-float
    const float r0 = rsqrtf(dot.hi);
    const ffx::ff h = ffx::ff_mul_f(ffx::ff_mul_f(dot, r0), r0);
    const ffx::ff r = ffx::ff_mul_f(ffx::ff_sub(ffx::ff_from(1.5f), ffx::ff_mul_f(h, 0.5f)), r0);
    if (scale <= 0x1p10f * sqrtf(dot.hi)) {
      for (int d = 0; d < 3; d++) {
        const ffx::ff x = ffx::ff_mul(nv3[d], r);
        n2[o + d] = make_float2(x.hi, x.lo);
      }
    } else {
      // the gradients cancel to below 2^-10 of their size: float64, as the reference
      const Normal64 nf = normal_f64(g, i, j, k, p[0], p[1], p[2], flip);
      for (int d = 0; d < 3; d++) {
        const ffx::ff x = ffx::ff_from_double(nf.n[d]);
        n2[o + d] = make_float2(x.hi, x.lo);
      }
      st.normal_f64++;
    }
  } else {
    float Gq[8][3];
#pragma unroll
    for (int q = 0; q < 8; q++)
      point_gradient_f(g, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1), (float*)G.inv2d, Gq[q]);
    float nv3[3];
    const float uu = p[0], vv = p[1], ww = p[2];
    const float sgn = flip ? -1.0f : 1.0f;
    float scale = 0;  // largest corner gradient component: the size of the interpolation's inputs
#pragma unroll
    for (int d = 0; d < 3; d++) {
#pragma unroll
      for (int q = 0; q < 8; q++) scale = fmaxf(scale, fabsf(Gq[q][d]));
      const float a0 = fmaf(uu, Gq[1][d] - Gq[0][d], Gq[0][d]), a1 = fmaf(uu, Gq[3][d] - Gq[2][d], Gq[2][d]);
      const float a2 = fmaf(uu, Gq[5][d] - Gq[4][d], Gq[4][d]), a3 = fmaf(uu, Gq[7][d] - Gq[6][d], Gq[6][d]);
      const float b0 = fmaf(vv, a1 - a0, a0), b1 = fmaf(vv, a3 - a2, a2);
      nv3[d] = sgn * fmaf(ww, b1 - b0, b0);
    }
    const float dot = nv3[0] * nv3[0] + nv3[1] * nv3[1] + nv3[2] * nv3[2];
    // The float32 interpolation errs by a few ulps of `scale`; where the gradients cancel to below
    // 1/16 of it (strongly uneven spacing, near critical points) that would exceed ~4e-6 of the
    // unit normal: the reference's float64 normal instead.
    if (scale <= 16.0f * sqrtf(dot)) {
      const float rn = rsqrtf(dot);
      for (int d = 0; d < 3; d++) out.n[o + d] = nv3[d] * rn;
    } else {
      const Normal64 nf = normal_f64(g, i, j, k, (double)p[0], (double)p[1], (double)p[2], flip);
      for (int d = 0; d < 3; d++) out.n[o + d] = (float)nf.n[d];
      st.normal_f64++;
    }
  }
  if (out.vcell) {
    out.vcell[vidx] = cell;
    out.vuvw[o] = p[0];
    out.vuvw[o + 1] = p[1];
    out.vuvw[o + 2] = p[2];
  }
}

__device__ __forceinline__ void flush_stats(const repr::Stats& st, unsigned long long* stats) {
  // representative counters (the reference's failed-projection counts) and float64 fallbacks
  if (st.fail1) atomicAdd(stats + 2, (unsigned long long)st.fail1);
  if (st.fail2) atomicAdd(stats + 3, (unsigned long long)st.fail2);
  if (st.fallback + st.normal_f64) atomicAdd(stats + 7, (unsigned long long)(st.fallback + st.normal_f64));
}

// One-pass vertex kernel over the vertices the two-pass kernels list (neighbour-contour exclusion,
// a distance that needs float64): the 7x7 projection with every float64 fallback.  Contours
// without a valid 7x7 sample go on to the tail list (the reference's 26x26 retry, one warp each).
// A list of at most `warp_max` entries is left whole to the warp kernel: one thread's serial
// projection (~0.1 ms) would set the latency of a small call.
__global__ void __launch_bounds__(kVertexThreads) dmc_vertex_kernel(CellSpace space, const uint16_t* cellof, const uint8_t* vrank,
                                                                     const uint32_t* vwork, const uint32_t* list,
                                                                     const unsigned* count, uint32_t* tail_list,
                                                                     unsigned* tail_count, unsigned warp_max,
                                                                     DmcVertexOut out, int flip_all,
                                                                     unsigned long long* stats) {
  __shared__ uint64_t cc[256];
  __shared__ float sample_lb[49 * kVertexThreads];  // per-thread sample bounds, column per thread
  const unsigned n = *count;
  if (n <= warp_max) return;
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  repr::Stats st;
  GridCache G;
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t vidx = (int64_t)list[a];
    const uint32_t vcell = slot_cell(cellof, vwork[vidx]);
    const int rank = vrank[vidx];
    G.load(space, vcell);
    const Grid& g = G.g;
    const int64_t cell = vcell - g.vbase;
    int i, j, k;
    cell_ijk(g, cell, i, j, k);
    VertexContour V;
    if (!vertex_contour(g, i, j, k, rank, cc, G.iso_ff, V)) continue;  // cannot happen: counted
    float p[3];
    int prj;
    if (!repr::representative_7x7(V.u, g.iso, V.c, V.tsel, V.pts + 3 * V.tstart, cnt_size(V.c, V.tsel), V.bx, p,
                                  st, sample_lb + threadIdx.x, kVertexThreads, prj)) {
      st.fail1++;
      tail_list[atomicAdd(tail_count, 1u)] = (uint32_t)vidx;
      continue;
    }
    vertex_outputs(G, i, j, k, cell, p, nullptr, vidx, out, flip_all | (g.flags & kGridFlip), st);
  }
  flush_stats(st, stats);
}

// warp-wide winner of the lanes' samples: smallest distance, then smallest loop index
__device__ __forceinline__ repr::LaneBest warp_best(repr::LaneBest b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    repr::LaneBest x;
    x.d = __shfl_xor_sync(0xffffffffu, b.d, o);
    x.w = __shfl_xor_sync(0xffffffffu, b.w, o);
    x.q = __shfl_xor_sync(0xffffffffu, b.q, o);
    if (repr::lane_better(x, b)) b = x;
  }
  return b;
}

// One warp per vertex: every lane rebuilds the contour and its projection frame (same cell, no
// divergence), the lanes split the samples, and lane 0 writes the outputs.  A listed vertex takes
// ~2 samples per lane for its 7x7 projection and ~22 for the reference's 26x26 retry, instead of up
// to 725 on one thread.  Work: the whole one-pass list when it has at most `warp_max` entries
// (the one-pass kernel then does nothing), otherwise the one-pass kernel's tail list.
__global__ void __launch_bounds__(kVertexThreads) dmc_vertex_warp_kernel(CellSpace space, const uint16_t* cellof, const uint8_t* vrank,
                                                                          const uint32_t* vwork, const uint32_t* list,
                                                                          const unsigned* count,
                                                                          const uint32_t* tail_list,
                                                                          const unsigned* tail_count,
                                                                          unsigned warp_max, DmcVertexOut out,
                                                                          int flip_all, unsigned long long* stats) {
  constexpr int kWarps = kVertexThreads / 32;
  __shared__ uint64_t cc[256];
  __shared__ float coords[kWarps][2][26];  // each warp's sample coordinates
  const bool whole = *count <= warp_max;   // 7x7 projections too, not only retries
  const uint32_t* L = whole ? list : tail_list;
  const int64_t n = whole ? (int64_t)*count : (int64_t)*tail_count;
  if (n == 0) return;
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* su = coords[wib][0];
  float* sv = coords[wib][1];
  repr::Stats st;
  GridCache G;
  int f64 = 0;
  for (int64_t a = (int64_t)blockIdx.x * kWarps + wib; a < n; a += (int64_t)gridDim.x * kWarps) {
    const int64_t vidx = (int64_t)L[a];
    const uint32_t vcell = slot_cell(cellof, vwork[vidx]);
    const int rank = vrank[vidx];
    G.load(space, vcell);
    const Grid& g = G.g;
    const int64_t cell = vcell - g.vbase;
    int i, j, k;
    cell_ijk(g, cell, i, j, k);
    VertexContour V;
    if (!vertex_contour(g, i, j, k, rank, cc, G.iso_ff, V)) continue;  // cannot happen (warp-uniform)
    const float* pts = V.pts + 3 * V.tstart;
    const int npts = cnt_size(V.c, V.tsel);
    repr::ProjCtx P;
    float us[7], vs[7];
    int f64c = 0;  // float64 sample coordinates: the same on every lane (counted once)
    repr::projection_setup(V.u, g.iso, V.c, V.tsel, pts, npts, V.bx, P, us, vs, f64c);
    if (whole && lane == 0) f64 += f64c;  // a retry's set-up was counted by the one-pass kernel
    repr::LaneBest b = repr::lane_none();
    int ns = 7;
    if (whole) {
      __syncwarp();  // the previous vertex's coordinates are no longer read
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 7; q++) {
          su[q] = us[q];
          sv[q] = vs[q];
        }
      }
      __syncwarp();
      b = warp_best(repr::grid_lane(P, su, sv, 7, lane, 32, pts, npts, f64));
      if (b.q == repr::kNoSample && lane == 0) st.fail1++;
    }
    if (b.q == repr::kNoSample) {
      // the reference's retry with 26x26 samples from the same mean point
      __syncwarp();
      if (lane < 26) {
        su[lane] = repr::tail_coord(V.bx.b[V.tsel][P.A][0], V.bx.b[V.tsel][P.A][1], lane + 1);
        sv[lane] = repr::tail_coord(V.bx.b[V.tsel][P.B][0], V.bx.b[V.tsel][P.B][1], lane + 1);
      }
      __syncwarp();
      b = warp_best(repr::grid_lane(P, su, sv, 26, lane, 32, pts, npts, f64));
      ns = 26;
    }
    if (lane == 0) {
      float p[3];
      if (b.q != repr::kNoSample) {
        repr::lane_point(P, su, sv, ns, b, p);
        vertex_outputs(G, i, j, k, cell, p, nullptr, vidx, out, flip_all | (g.flags & kGridFlip), st);
      } else {
        // nothing valid at 26x26 either: the reference keeps its float64 mean point, unrounded
        st.fail2++;
        const repr::Point64 pm = repr::mean_point_exact(pts, npts);
        for (int d = 0; d < 3; d++) p[d] = (float)pm.p[d];
        const bool exact = (double)p[0] == pm.p[0] && (double)p[1] == pm.p[1] && (double)p[2] == pm.p[2];
        vertex_outputs(G, i, j, k, cell, p, exact ? nullptr : pm.p, vidx, out, flip_all | (g.flags & kGridFlip),
                       st);
      }
    }
  }
  st.fallback += f64;
  flush_stats(st, stats);
}

// Two-pass vertices, pass 1: contour, plane, sample coordinates, mean point -> one record per
// vertex.  Only the vertex's own contour is evaluated: its edge points are summed and boxed as they
// are computed (no point array, nothing in local memory).  Contours with neighbour-contour
// exclusion go to the one-pass kernel's list.
__global__ void __launch_bounds__(kVertexThreads, 5) dmc_vertex_setup_kernel(CellSpace space, const uint16_t* cellof, const uint8_t* vrank,
                                                                              const uint32_t* vwork, int64_t nv,
                                                                              repr::ProjRecord* recs, uint32_t* list,
                                                                              unsigned* count,
                                                                              unsigned long long* stats) {
  __shared__ uint64_t cc[256];
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  GridCache G;
  int f64 = 0;
  for (int64_t vidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vidx < nv;
       vidx += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t vcell = slot_cell(cellof, vwork[vidx]);
    const int rank = vrank[vidx];
    G.load(space, vcell);
    const Grid& g = G.g;
    int i, j, k;
    cell_ijk(g, vcell - g.vbase, i, j, k);
    float u[8];
    load_corners(g, i, j, k, u);
    const uint64_t c = dmc_polygon(mc_case(u, g.iso_up), u, g.iso, cc);
    // the rank-th used contour (one with an interior edge), as vertex_contour selects it
    const int ncnt = cnt_count(c);
    int flat = 0, seen = 0, tsel = -1, tstart = 0;
    for (int t = 0; t < ncnt && tsel < 0; t++) {
      const int sz = cnt_size(c, t);
      bool used = false;
      for (int q = 0; q < sz; q++) used = used || edge_interior(g, i, j, k, cnt_edge(c, flat + q));
      if (used) {
        if (seen == rank) {
          tsel = t;
          tstart = flat;
        }
        seen++;
      }
      flat += sz;
    }
    repr::ProjRecord& R = recs[vidx];  // written in place: no copy in local memory
    bool ok = tsel >= 0;              // cannot fail: counted
    if (ok) {
      const int n = cnt_size(c, tsel);
      repr::ContourAcc A;
      repr::contour_acc(u, g.iso, G.iso_ff, c, tstart, n, A);
      int f64c = 0;
      ok = repr::projection_record_acc(u, g.iso, c, tsel, tstart, n, A, R, f64c);
      if (ok) f64 += f64c;  // contours redone by the one-pass kernel are counted there
    }
    if (!ok) {
      R.prj = -1;
      list[atomicAdd(count, 1u)] = (uint32_t)vidx;
    }
  }
  if (f64) atomicAdd(stats + 7, (unsigned long long)f64);
}

// Two-pass vertices, pass 2: the projection from the record.  p (local coordinates) goes to vp;
// vertices that need float64 go to the one-pass kernel's list (vp.w = 1 marks them).
__global__ void __launch_bounds__(kVertexThreads) dmc_project_kernel(const repr::ProjRecord* recs, int64_t nv,
                                                                     float4* vp, uint32_t* list, unsigned* count,
                                                                     unsigned long long* stats) {
  __shared__ float sample_lb[49 * kVertexThreads];
  int f64 = 0;
  for (int64_t vidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vidx < nv;
       vidx += (int64_t)gridDim.x * blockDim.x) {
    const repr::ProjRecord& R = recs[vidx];
    if (R.prj < 0) {  // already listed by the set-up pass
      vp[vidx] = make_float4(0, 0, 0, 1);
      continue;
    }
    float p[3] = {0, 0, 0};
    int f = 0;
    const int r = repr::projection_from_record(R, p, sample_lb + threadIdx.x, kVertexThreads, f);
    if (r != 0) list[atomicAdd(count, 1u)] = (uint32_t)vidx;  // redone (and counted) by the one-pass kernel
    else f64 += f;
    vp[vidx] = make_float4(p[0], p[1], p[2], r != 0 ? 1.0f : 0.0f);
  }
  if (f64) atomicAdd(stats + 7, (unsigned long long)f64);
}

// Two-pass vertices, pass 2 for small meshes: G lanes per record (G a power of two, 2..32) split
// its 49 samples, so that a call's latency is that of ~49/G exact samples instead of one thread's
// serial projection.  Same outputs and lists as dmc_project_kernel.
__global__ void __launch_bounds__(kVertexThreads) dmc_project_group_kernel(const repr::ProjRecord* recs, int64_t nv,
                                                                           int G, float4* vp, uint32_t* list,
                                                                           unsigned* count,
                                                                           unsigned long long* stats) {
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const int64_t per_warp = 32 / G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int f64 = 0;
  // base is the same on every lane of a warp, so all lanes reach the shuffles
  for (int64_t base = warp * per_warp; base < nv; base += nwarps * per_warp) {
    const int64_t vidx = base + lane / G;
    const bool valid = vidx < nv;
    const repr::ProjRecord& R = recs[valid ? vidx : base];
    const bool listed = R.prj < 0;  // already listed by the set-up pass (same for the whole group)
    repr::LaneBest b = repr::lane_none();
    bool unc = false;
    repr::ProjCtx P;
    if (valid && !listed) {
      repr::ctx_from_record(R, P);
      b = repr::record_lane(P, R, gl, G, f64, unc);
    }
    for (int o = G >> 1; o > 0; o >>= 1) {
      repr::LaneBest x;
      x.d = __shfl_xor_sync(0xffffffffu, b.d, o);
      x.w = __shfl_xor_sync(0xffffffffu, b.w, o);
      x.q = __shfl_xor_sync(0xffffffffu, b.q, o);
      unc = __shfl_xor_sync(0xffffffffu, (int)unc, o) != 0 || unc;
      if (repr::lane_better(x, b)) b = x;
    }
    if (!valid || gl != 0) continue;
    if (listed) {
      vp[vidx] = make_float4(0, 0, 0, 1);
    } else if (unc || b.q == repr::kNoSample) {
      list[atomicAdd(count, 1u)] = (uint32_t)vidx;  // redone (and counted) by the one-pass kernels
      vp[vidx] = make_float4(0, 0, 0, 1);
    } else {
      float p[3];
      repr::lane_point(P, R.us, R.vs, 7, b, p);
      vp[vidx] = make_float4(p[0], p[1], p[2], 0.0f);
    }
  }
  if (f64) atomicAdd(stats + 7, (unsigned long long)f64);
}

// Two-pass vertices, pass 3: positions, normals and local coordinates of the projected vertices.
template <bool kFF>
__global__ void __launch_bounds__(kVertexThreads, 4) dmc_vertex_finish_kernel(CellSpace space, const uint16_t* cellof,
                                                                            const uint32_t* vwork,
                                                                            int64_t nv, const float4* vp,
                                                                            DmcVertexOut out, int flip_all,
                                                                            unsigned long long* stats) {
  repr::Stats st;
  GridCache G;
  for (int64_t vidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vidx < nv;
       vidx += (int64_t)gridDim.x * blockDim.x) {
    const float4 q = vp[vidx];
    if (q.w != 0.0f) continue;  // done by the one-pass kernel
    const uint32_t vcell = slot_cell(cellof, vwork[vidx]);
    G.load(space, vcell);
    const Grid& g = G.g;
    const int64_t cell = vcell - g.vbase;
    int i, j, k;
    cell_ijk(g, cell, i, j, k);
    const float p[3] = {q.x, q.y, q.z};
    vertex_outputs<kFF>(G, i, j, k, cell, p, nullptr, vidx, out, flip_all | (g.flags & kGridFlip), st);
  }
  flush_stats(st, stats);
}

// ------------------------------------------------------------------------------------------
// quads: the cell owning a crossed interior edge (its edge 0, 3 or 8) gathers the vertices of the
// four cells around it.  Slot by the side of the edge's first end vertex (get_vertex_pos,
// cpp_dmc/DualMarchingCubes.h:221-224); colour 3*parity(i,j,k) + axis (:177-180).
// ------------------------------------------------------------------------------------------
// Quad corners are vertex indices within the quad's own volume: the space-wide offsets minus the
// volume's first vertex (the scanned tile offset of its first tile; 0 for a single volume).
// The quads a cell owns (one per crossed interior edge 0, 3, 8), from the records of the four
// cells around each edge (listed cells: a crossed edge makes every cell around it listed).
__device__ __forceinline__ void cell_quads(const Grid& g, int32_t vfirst, uint32_t slot, int64_t vc, unsigned cs,
                                           const CellMask* mask, const uint32_t* rec, const int32_t* voff,
                                           const int32_t* qoff, int32_t* quads, uint8_t* colors) {
  // cell offsets (di, dj, dk) and local edge of the four cells around the owned edges 0, 3, 8
  // x edge: (0,-1,-1) e6, (0,0,-1) e4, (0,-1,0) e2, (0,0,0) e0
  // y edge: (-1,0,-1) e5, (0,0,-1) e7, (-1,0,0) e1, (0,0,0) e3
  // z edge: (-1,-1,0) e10, (0,-1,0) e11, (-1,0,0) e9, (0,0,0) e8
  const int64_t cell = vc - g.vbase;
  int i, j, k;
  cell_ijk(g, cell, i, j, k);
  // from the cell's MC case (bit v: corner v at or above the isovalue): corner 0's side, and the
  // crossings of edges 0 (corners 0-1), 3 (0-2) and 8 (0-4)
  const int neg = !(cs & 1u);  // first end vertex below the isovalue
  const bool crossed[3] = {((cs ^ (cs >> 1)) & 1u) != 0, ((cs ^ (cs >> 2)) & 1u) != 0, ((cs ^ (cs >> 4)) & 1u) != 0};
  int32_t q = qoff[slot];
  const int par = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!crossed[a] || !edge_interior(g, i, j, k, a == 0 ? 0 : (a == 1 ? 3 : 8))) continue;
    int di[4], dj[4], dk[4], le[4];
    if (a == 0) {
      di[0] = 0; dj[0] = -1; dk[0] = -1; le[0] = 6;
      di[1] = 0; dj[1] = 0; dk[1] = -1; le[1] = 4;
      di[2] = 0; dj[2] = -1; dk[2] = 0; le[2] = 2;
      di[3] = 0; dj[3] = 0; dk[3] = 0; le[3] = 0;
    } else if (a == 1) {
      di[0] = -1; dj[0] = 0; dk[0] = -1; le[0] = 5;
      di[1] = 0; dj[1] = 0; dk[1] = -1; le[1] = 7;
      di[2] = -1; dj[2] = 0; dk[2] = 0; le[2] = 1;
      di[3] = 0; dj[3] = 0; dk[3] = 0; le[3] = 3;
    } else {
      di[0] = -1; dj[0] = -1; dk[0] = 0; le[0] = 10;
      di[1] = 0; dj[1] = -1; dk[1] = 0; le[1] = 11;
      di[2] = -1; dj[2] = 0; dk[2] = 0; le[2] = 9;
      di[3] = 0; dj[3] = 0; dk[3] = 0; le[3] = 8;
    }
    int32_t qv[4];
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const uint32_t ns = s == 3 ? slot : listed_slot(mask, (uint32_t)g.vcell(i + di[s], j + dj[s], k + dk[s]));
      const uint32_t rn = rec[ns];
      qv[quad_slot(le[s], neg)] = voff[ns] - vfirst + rec_rank(rn, le[s]);
    }
    reinterpret_cast<int4*>(quads)[q] = make_int4(qv[0], qv[1], qv[2], qv[3]);
    if (colors) colors[q] = (uint8_t)(3 * par + a);
    q++;
  }
}

// Each warp walks chunks of 32 consecutive slots of the listed cells, queues those that own quads
// (ballot) in shared memory and processes the queue 32 cells at a time, one per lane.  No block
// barrier.
constexpr int kQuadThreads = 256;
template <bool kBatch>
__global__ void __launch_bounds__(kQuadThreads) dmc_quad_kernel(CellSpace space, const CellMask* mask,
                                                                const uint16_t* cellof, const uint8_t* ccase,
                                                                const uint32_t* rec,
                                                                const int32_t* voff, const int32_t* qoff,
                                                                const unsigned long long* tile_off, int32_t* quads,
                                                                uint8_t* colors) {
  constexpr int kWarps = kQuadThreads / 32;
  __shared__ uint32_t queue[kWarps][64];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t* Q = queue[wid];
  const int64_t tiles = ceil_div(space.n, kScanTile), chunks = tiles * (kScanTile / 32);
  int qn = 0;  // queued cells (the same on every lane)
  for (int64_t chunk = (int64_t)blockIdx.x * kWarps + wid;; chunk += (int64_t)gridDim.x * kWarps) {
    const bool more = chunk < chunks;
    if (more) {
      int64_t tile;
      uint32_t first;
      slot_chunk(chunk, tiles, tile, first);
      const uint32_t slot = first + lane, r = slot & (kScanTile - 1);
      const bool own = r < tile_listed(mask, tile) && rec_nq(rec[slot]) != 0;
      const unsigned bal = __ballot_sync(0xffffffffu, own);
      if (own) Q[qn + __popc(bal & ((1u << lane) - 1u))] = slot;
      qn += __popc(bal);
      __syncwarp();
    }
    while (qn >= 32 || (!more && qn > 0)) {
      const int take = qn < 32 ? qn : 32;
      if (lane < take) {
        const uint32_t slot = Q[lane];
        const uint32_t vc = slot_cell(cellof, slot);
        const Grid& g = kBatch ? space.grids[__ldg(space.tile_vol + vc / kScanTile)] : space.one;
        const int32_t vfirst = kBatch ? (int32_t)(tile_off[g.vbase / kScanTile] >> 32) : 0;
        cell_quads(g, vfirst, slot, vc, __ldg(ccase + slot), mask, rec, voff, qoff, quads, colors);
      }
      __syncwarp();
      const int rest = qn - take;  // at most 31: move them to the front
      const uint32_t x = lane < rest ? Q[take + lane] : 0u;
      __syncwarp();
      if (lane < rest) Q[lane] = x;
      __syncwarp();
      qn = rest;
    }
    if (!more) break;
  }
}

// ------------------------------------------------------------------------------------------
// host-side launches
// ------------------------------------------------------------------------------------------
int dmc_front_count(const CellSpace& space, DmcScratch& s, cudaStream_t st, Prof* prof, const TileGate* gates,
                    int ngates) {
  const int64_t tiles = ceil_div(space.n, kScanTile);
  int k = 0, dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  {
    Stage t(prof, "dmc_classify", st);
    // the ambiguous cells' list lives in qoff until the offsets kernel writes the quad offsets
    cudaMemsetAsync(s.amb_n, 0, sizeof(unsigned), st);
    auto classify = [&](int64_t t0, int64_t t1) {
      if (t1 <= t0) return;
      if (space.one.gen)  // fused generation (single volumes)
        dmc_classify_kernel<true><<<(unsigned)(t1 - t0), kScanThreads, 0, st>>>(
            space, t0, s.rec, s.cellof, s.ccase, s.mask, s.tile_sums, s.stats, reinterpret_cast<uint32_t*>(s.qoff), s.amb_n);
      else
        dmc_classify_kernel<false><<<(unsigned)(t1 - t0), kScanThreads, 0, st>>>(
            space, t0, s.rec, s.cellof, s.ccase, s.mask, s.tile_sums, s.stats, reinterpret_cast<uint32_t*>(s.qoff), s.amb_n);
      k++;
    };
    if (ngates == 0) classify(0, tiles);
    int64_t t0 = 0;
    for (int q = 0; q < ngates; q++) {
      cudaStreamWaitEvent(st, gates[q].ready, 0);
      const int64_t t1 = (q == ngates - 1) ? tiles : std::min(gates[q].tile_end, tiles);
      classify(t0, t1);
      t0 = std::max(t0, t1);
    }
    // one wave; the list length is only known on the device, so the grid follows the cell count
    static const int r_amb = resident_blocks(dmc_amb_kernel, 128);
    dmc_amb_kernel<<<(unsigned)wave_grid(r_amb, sms, 16, ceil_div(space.n, 128), 128), 128, 0, st>>>(
        space, s.cellof, s.rec, s.tile_sums, reinterpret_cast<const uint32_t*>(s.qoff), s.amb_n);
    k++;
  }
  Stage t(prof, "dmc_scan", st);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(s.tile_sums, tiles, s.totals);
  return k + 1;
}

int64_t dmc_tiles(const CellSpace& space) { return ceil_div(space.n, kScanTile); }

int dmc_front_emit(const CellSpace& space, DmcScratch& s, DmcVertexOut vo, int64_t nv, int32_t* quads,
                   uint8_t* colors, int flip, const Tuning& tu, cudaStream_t st, Prof* prof) {
  const int sms = tu.sms;
  const int64_t n = space.n;
  {
    // per-cell offsets and the vertex work list (needs the vertex count for its size)
    Stage t(prof, "dmc_scan", st);
    const int64_t tiles = ceil_div(n, kScanTile);
    dmc_offsets_kernel<<<(unsigned)ceil_div(tiles, kOffsetWarps), 32 * kOffsetWarps, 0, st>>>(
        s.mask, s.rec, s.tile_sums, tiles, s.voff, s.qoff, s.vwork, s.vrank);
  }
  // per-vertex grids: whole waves of each kernel's resident blocks
  static const int r_setup = resident_blocks(dmc_vertex_setup_kernel, kVertexThreads);
  static const int r_project = resident_blocks(dmc_project_kernel, kVertexThreads);
  static const int r_finish = resident_blocks(dmc_vertex_finish_kernel<true>, kVertexThreads);
  static const int r_finish32 = resident_blocks(dmc_vertex_finish_kernel<false>, kVertexThreads);
  static const int r_quad = resident_blocks(dmc_quad_kernel<false>, kQuadThreads);
  static const int r_quad_batch = resident_blocks(dmc_quad_kernel<true>, kQuadThreads);
  auto vgrid = [&](int resident) {
    return (unsigned)wave_grid(resident, sms, tu.vertex_blocks_per_sm, nv, kVertexThreads);
  };
  {
    Stage t(prof, "dmc_vertex_setup", st);
    cudaMemsetAsync(s.fb_count, 0, 2 * sizeof(unsigned), st);
    dmc_vertex_setup_kernel<<<vgrid(r_setup), kVertexThreads, 0, st>>>(space, s.cellof, s.vrank, s.vwork, nv, s.proj, s.fb_list,
                                                                       s.fb_count, s.stats);
  }
  {
    Stage t(prof, "dmc_project", st);
    // lanes per record: as many as the tuning's lane budget allows (small meshes), else one thread
    int G = 1;
    while (G < 32 && nv * G * 2 <= tu.group_lanes) G *= 2;
    if (G >= 4)
      dmc_project_group_kernel<<<(unsigned)std::max<int64_t>(1, ceil_div(nv * G, kVertexThreads)), kVertexThreads, 0,
                                 st>>>(s.proj, nv, G, s.vp, s.fb_list, s.fb_count, s.stats);
    else
      dmc_project_kernel<<<vgrid(r_project), kVertexThreads, 0, st>>>(s.proj, nv, s.vp, s.fb_list, s.fb_count, s.stats);
  }
  {
    Stage t(prof, "dmc_vertex_finish", st);
    // the float-float normals only when some volume keeps float64 normals (simplification)
    if (vo.n64)
      dmc_vertex_finish_kernel<true><<<vgrid(r_finish), kVertexThreads, 0, st>>>(space, s.cellof, s.vwork, nv, s.vp, vo, flip,
                                                                                 s.stats);
    else
      dmc_vertex_finish_kernel<false><<<vgrid(r_finish32), kVertexThreads, 0, st>>>(space, s.cellof, s.vwork, nv, s.vp, vo, flip,
                                                                                    s.stats);
  }
  {
    // the listed vertices: one thread each with every float64 fallback, the 26x26 retries one warp
    // each; a short list (small calls) entirely one warp per vertex
    Stage t(prof, "dmc_vertex", st);
    const unsigned warp_max = (unsigned)std::min<int64_t>(tu.warp_list_max, 0x7fffffff);
    static const int r_vertex = resident_blocks(dmc_vertex_kernel, kVertexThreads);
    const unsigned fb = (unsigned)wave_grid(r_vertex, sms, 8, nv, kVertexThreads);
    dmc_vertex_kernel<<<fb, kVertexThreads, 0, st>>>(space, s.cellof, s.vrank, s.vwork, s.fb_list, s.fb_count, s.tail_list,
                                                      s.fb_count + 1, warp_max, vo, flip, s.stats);
    dmc_vertex_warp_kernel<<<(unsigned)std::max(1, sms * 3), kVertexThreads, 0, st>>>(
        space, s.cellof, s.vrank, s.vwork, s.fb_list, s.fb_count, s.tail_list, s.fb_count + 1, warp_max, vo, flip,
        s.stats);
  }
  Stage t(prof, "dmc_quad", st);
  // one wave: the kernel takes 32-cell chunks until none are left
  if (space.grids)
    dmc_quad_kernel<true><<<(unsigned)wave_grid(r_quad_batch, sms, tu.quad_blocks_per_sm, ceil_div(n, 32),
                                                kQuadThreads / 32), kQuadThreads,
                            0, st>>>(space, s.mask, s.cellof, s.ccase, s.rec, s.voff, s.qoff, s.tile_sums, quads, colors);
  else
    dmc_quad_kernel<false><<<(unsigned)wave_grid(r_quad, sms, tu.quad_blocks_per_sm, ceil_div(n, 32),
                                                 kQuadThreads / 32), kQuadThreads, 0,
                             st>>>(space, s.mask, s.cellof, s.ccase, s.rec, s.voff, s.qoff, s.tile_sums, quads,
                                   colors);
  return 7;
}

}  // namespace tmc
