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
//   dmc_vertex_kernel    vertex representatives (cpp_dmc representative/projection), normals,
//                        positions
//   dmc_quad_kernel      each cell emits the quads of its crossed interior edges 0, 3, 8 by
//                        looking up the four cells around the edge
#include <cstdio>

#include "common.cuh"
#include "dmc.h"
#include "scan.cuh"

namespace tmc {

__constant__ uint64_t c_case_contour[256] = TMC_CASE_CONTOUR_INIT;

// per-cell record
//   bits 0-2   nV: used contours (vertices this cell emits)
//   bits 3-4   nQ: crossed interior edges among the cell's edges 0, 3, 8 (quads it owns)
//   bits 5-28  for each edge e, 2 bits: rank of the used contour holding e
//   bit  29    ambiguous case
__device__ __forceinline__ int rec_nv(uint32_t r) { return r & 7; }
__device__ __forceinline__ int rec_nq(uint32_t r) { return (r >> 3) & 3; }
__device__ __forceinline__ int rec_rank(uint32_t r, int e) { return (r >> (5 + 2 * e)) & 3; }

__device__ __forceinline__ bool edge_interior(const Grid& g, int i, int j, int k, int e) {
  const int off = edge_off(e), ax = edge_axis(e);
  const int gi = i + (off & 1), gj = j + ((off >> 1) & 1), gk = k + ((off >> 2) & 1);
  bool ok = true;
  if (ax != 0) ok = ok && gi >= 1 && gi <= g.nx - 2;
  if (ax != 1) ok = ok && gj >= 1 && gj <= g.ny - 2;
  if (ax != 2) ok = ok && gk >= 1 && gk <= g.nz - 2;
  return ok;
}

__device__ __forceinline__ void load_corners(const Grid& g, int i, int j, int k, float u[8]) {
  const float* p = g.f + ((int64_t)k * g.ny + j) * g.nx + i;
  const int64_t sy = g.nx, sz = (int64_t)g.nx * g.ny;
  u[0] = __ldg(p);
  u[1] = __ldg(p + 1);
  u[2] = __ldg(p + sy);
  u[3] = __ldg(p + sy + 1);
  u[4] = __ldg(p + sz);
  u[5] = __ldg(p + sz + 1);
  u[6] = __ldg(p + sz + sy);
  u[7] = __ldg(p + sz + sy + 1);
}

__device__ __forceinline__ unsigned mc_case(const float u[8], float iso_up) {
  unsigned c = 0;
#pragma unroll
  for (int v = 0; v < 8; v++) c |= (unsigned)(u[v] >= iso_up) << v;
  return c;
}

// Linear cell index -> (i, j, k)
__device__ __forceinline__ void cell_ijk(const Grid& g, int64_t c, int& i, int& j, int& k) {
  const int64_t cx = g.nx - 1, cy = g.ny - 1;
  i = (int)(c % cx);
  const int64_t r = c / cx;
  j = (int)(r % cy);
  k = (int)(r / cy);
}

// ------------------------------------------------------------------------------------------
// classification
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t classify_cell(const Grid& g, int i, int j, int k, const uint64_t* cc,
                                                  unsigned long long* stats) {
  float u[8];
  load_corners(g, i, j, k, u);
  const unsigned cs = mc_case(u, g.iso_up);
  if (cs == 0 || cs == 255) return 0;
  const bool amb = case_ambiguous(cs);
  const uint64_t c = dmc_polygon(cs, u, g.iso, cc);
  const int ncnt = cnt_count(c);
  uint32_t rec = amb ? (1u << 29) : 0u;
  int nv = 0, flat = 0;
  for (int t = 0; t < ncnt; t++) {
    const int sz = cnt_size(c, t);
    bool used = false;
    for (int q = 0; q < sz; q++) used = used || edge_interior(g, i, j, k, cnt_edge(c, flat + q));
    if (used) {
      for (int q = 0; q < sz; q++) rec |= (uint32_t)nv << (5 + 2 * cnt_edge(c, flat + q));
      nv++;
    }
    flat += sz;
  }
  // owned quads: crossed interior edges 0 (x), 3 (y), 8 (z) at the cell's lower corner
  const uint32_t em = case_edge_mask(cs);
  int nq = 0;
  nq += ((em >> 0) & 1) && edge_interior(g, i, j, k, 0);
  nq += ((em >> 3) & 1) && edge_interior(g, i, j, k, 3);
  nq += ((em >> 8) & 1) && edge_interior(g, i, j, k, 8);
  rec |= (uint32_t)nv | ((uint32_t)nq << 3);
  (void)stats;
  return rec;
}

// One block handles kScanTile consecutive cells (linear order), writes their records and the
// tile's packed (vertices << 32 | quads) sum.
__global__ void __launch_bounds__(kScanThreads) dmc_classify_kernel(Grid g, uint32_t* rec,
                                                                   unsigned long long* tile_sums,
                                                                   unsigned long long* stats) {
  __shared__ uint64_t cc[256];
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  const int64_t n = g.ncells();
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  unsigned long long local = 0, act = 0, amb = 0;
  for (int s = 0; s < kScanItems; s++) {
    const int64_t c = base + (int64_t)s * kScanThreads + threadIdx.x;
    if (c >= n) break;
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const uint32_t r = classify_cell(g, i, j, k, cc, stats);
    rec[c] = r;
    local += ((unsigned long long)rec_nv(r) << 32) | (unsigned long long)rec_nq(r);
    act += r != 0;
    amb += (r >> 29) & 1;
  }
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(local, &tot);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
  // statistics: active and ambiguous cells
  for (int o = 16; o; o >>= 1) {
    act += __shfl_down_sync(0xffffffffu, act, o);
    amb += __shfl_down_sync(0xffffffffu, amb, o);
  }
  if ((threadIdx.x & 31) == 0 && (act | amb)) {
    atomicAdd(stats + 0, act);
    atomicAdd(stats + 1, amb);
  }
}

// In-tile exclusive scan of the records -> per-cell vertex and quad offsets.
__global__ void __launch_bounds__(kScanThreads) dmc_offsets_kernel(int64_t n, const uint32_t* rec,
                                                                  const unsigned long long* tile_off,
                                                                  int32_t* voff, int32_t* qoff) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  // thread t owns cells base + t*kScanItems .. + kScanItems-1 (contiguous) for the scan
  uint32_t r[kScanItems];
  unsigned long long local = 0;
  const int64_t mine = base + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    r[s] = (mine + s < n) ? rec[mine + s] : 0u;
    local += ((unsigned long long)rec_nv(r[s]) << 32) | (unsigned long long)rec_nq(r[s]);
  }
  unsigned long long tot;
  unsigned long long pre = block_exclusive_scan<unsigned long long>(local, &tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int s = 0; s < kScanItems; s++) {
    if (mine + s < n) {
      voff[mine + s] = (int32_t)(pre >> 32);
      qoff[mine + s] = (int32_t)(pre & 0xffffffffull);
    }
    pre += ((unsigned long long)rec_nv(r[s]) << 32) | (unsigned long long)rec_nq(r[s]);
  }
}

// ------------------------------------------------------------------------------------------
// vertex representative: exact restatement of the reference's mixed float/double arithmetic
// (representative / projection, cpp_dmc/DualMarchingCubes.cpp:194-326).  The library is built
// with -fmad=false, so each line below rounds exactly like the CPU code.
// ------------------------------------------------------------------------------------------
struct CellBoxes {
  float b[4][3][2];  // contour, axis, min/max (values are floats; compared as doubles)
};

// getLocalCoordinates (cpp_dmc/DualMarchingCubes.h:391-407)
__device__ __forceinline__ void local_coord(int e, const float u[8], double iso, float out[3]) {
  const int v0 = edge_v0(e), v1 = edge_v1(e);
  const float l = (iso - (double)u[v0]) / ((double)u[v1] - (double)u[v0]);
  const int ax = edge_axis(e), con = edge_off(e);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float val = (d == ax) ? 1.0f : 0.0f;
    const float cn = (float)((con >> d) & 1);
    out[d] = l * val + cn;
  }
}

// isInNeighborBBox (cpp_dmc/DualMarchingCubes.h:498-517) with the projection's axis order
__device__ __forceinline__ bool in_neighbor_bbox(double u, double v, double w, uint64_t c, int t,
                                                 const CellBoxes& bx, int A, int B, int W) {
  const int ncnt = cnt_count(c);
  for (int i = 0; i < ncnt; i++) {
    if (cnt_size(c, i) == 3 && t != i) {
      if (u < (double)bx.b[i][A][0] || (double)bx.b[i][A][1] < u) continue;
      if (v < (double)bx.b[i][B][0] || (double)bx.b[i][B][1] < v) continue;
      if (w < (double)bx.b[i][W][0] || (double)bx.b[i][W][1] < w) continue;
      return true;
    }
  }
  return false;
}

// projection (cpp_dmc/DualMarchingCubes.cpp:274-326).  Plane pr: 0 = w (z), 1 = v (y), 2 = u (x).
// The corner permutation of the plane is applied to the field values by the caller (fp).
__device__ bool projection_exact(const double fp[8], double iso, uint64_t c, int t, double p[3],
                                 const CellBoxes& bx, int A, int B, int W, int nrSamples) {
  const double umin = bx.b[t][A][0], umax = bx.b[t][A][1];
  const double vmin = bx.b[t][B][0], vmax = bx.b[t][B][1];
  const double du = (umax - umin) / (nrSamples - 1);
  const double dv = (vmax - vmin) / (nrSamples - 1);
  double minDistance = 100;
  double pt0 = 0, pt1 = 0, pt2 = -1;
  double wmin = bx.b[t][W][0], wmax = bx.b[t][W][1];
  const double eps = 1e-5;
  if (fabs(wmax - wmin) < eps) {
    wmin -= eps;
    wmax += eps;
  }
  const int cnt = cnt_count(c);
  const int cnt_sz = cnt_size(c, t);
  for (int i = 1; i < (nrSamples - 1); i++) {
    const float u = umin + i * du;
    for (int j = 1; j < (nrSamples - 1); j++) {
      const float v = vmin + j * dv;
      const float g1 = (1 - v) * ((1 - u) * fp[0] + u * fp[1]) + v * ((1 - u) * fp[2] + u * fp[3]);
      const float g2 = (1 - v) * ((1 - u) * fp[4] + u * fp[5]) + v * ((1 - u) * fp[6] + u * fp[7]);
      if (g1 == g2) continue;
      const float w = (iso - g1) / (g2 - g1);
      if (wmin <= w && w <= wmax) {
        if (cnt == 1 || cnt_sz == 3 || !in_neighbor_bbox(u, v, w, c, t, bx, A, B, W)) {
          const float d = (p[0] - u) * (p[0] - u) + (p[1] - v) * (p[1] - v) + (p[2] - w) * (p[2] - w);
          if (minDistance > d) {
            minDistance = d;
            pt0 = u;
            pt1 = v;
            pt2 = w;
          }
        }
      }
    }
  }
  if (pt2 > -1) {
    p[0] = pt0;
    p[1] = pt1;
    p[2] = pt2;
    return true;
  }
  return false;
}

// representative (cpp_dmc/DualMarchingCubes.cpp:194-272)
__device__ void representative_exact(const float u[8], double iso, uint64_t c, int t, double p[3],
                                     const CellBoxes& bx, unsigned long long* stats) {
  int prj = 0;  // 0 = W, 1 = V, 2 = U
  double f[8];
#pragma unroll
  for (int q = 0; q < 8; q++) f[q] = u[q];
  if (cnt_size(c, t) >= 6) {
    const double uu = p[0], vv = p[1], ww = p[2];
    const double g0 = (1 - ww) * ((1 - vv) * (f[1] - f[0]) + vv * (f[3] - f[2])) + ww * ((1 - vv) * (f[5] - f[4]) + vv * (f[7] - f[6]));
    const double g1 = (1 - ww) * ((1 - uu) * (f[2] - f[0]) + uu * (f[3] - f[1])) + ww * ((1 - uu) * (f[6] - f[4]) + uu * (f[7] - f[5]));
    const double g2 = (1 - vv) * ((1 - uu) * (f[4] - f[0]) + uu * (f[5] - f[1])) + vv * ((1 - uu) * (f[6] - f[2]) + uu * (f[7] - f[3]));
    const double dx = fabs(g0), dy = fabs(g1), dz = fabs(g2);
    if (dz >= dx && dz >= dy) prj = 0;
    else if (dy >= dx && dy >= dz) prj = 1;
    else if (dx >= dy && dx >= dz) prj = 2;
    else prj = 0;
  } else {
    const double su = (double)bx.b[t][0][1] - (double)bx.b[t][0][0];
    const double sv = (double)bx.b[t][1][1] - (double)bx.b[t][1][0];
    const double sw = (double)bx.b[t][2][1] - (double)bx.b[t][2][0];
    if (sw <= su && sw <= sv) prj = 0;
    else if (sv <= su && sv <= sw) prj = 1;
    else if (su <= sv && su <= sw) prj = 2;
    else prj = 0;
  }
  // plane axes (A, B, W) and the corner permutation of the plane (w_proj / v_proj / u_proj)
  int A, B, W;
  uint32_t perm;
  if (prj == 0) { A = 0; B = 1; W = 2; perm = 0x76543210u; }
  else if (prj == 1) { A = 0; B = 2; W = 1; perm = 0x76325410u; }
  else { A = 1; B = 2; W = 0; perm = 0x75316420u; }
  double fp[8];
#pragma unroll
  for (int q = 0; q < 8; q++) fp[q] = f[(perm >> (4 * q)) & 0xF];
  double pt[3] = {p[A], p[B], p[W]};
  if (!projection_exact(fp, iso, c, t, pt, bx, A, B, W, 9)) {
    atomicAdd(stats + 2, 1ull);
    if (!projection_exact(fp, iso, c, t, pt, bx, A, B, W, 28)) atomicAdd(stats + 3, 1ull);
  }
  p[A] = pt[0];
  p[B] = pt[1];
  p[W] = pt[2];
}

// estimateGradient at a grid point (cpp_dmc/UniformGrid.cpp:512-540): central differences with
// the reference's border indexing ((i<0) ? 0 : (i>=max) ? max-i : i).
__device__ __forceinline__ int grad_index(int i, int max) { return (i < 0) ? 0 : (i >= max) ? max - i : i; }
__device__ __forceinline__ void point_gradient(const Grid& g, int i, int j, int k, double out[3]) {
  const int i0 = grad_index(i - 1, g.nx), i1 = grad_index(i + 1, g.nx);
  const int j0 = grad_index(j - 1, g.ny), j1 = grad_index(j + 1, g.ny);
  const int k0 = grad_index(k - 1, g.nz), k1 = grad_index(k + 1, g.nz);
  out[0] = ((double)g.at(i1, j, k) - (double)g.at(i0, j, k)) / (2 * g.dx);
  out[1] = ((double)g.at(i, j1, k) - (double)g.at(i, j0, k)) / (2 * g.dy);
  out[2] = ((double)g.at(i, j, k1) - (double)g.at(i, j, k0)) / (2 * g.dz);
}

__global__ void __launch_bounds__(128) dmc_vertex_kernel(Grid g, const uint32_t* rec, const int32_t* voff,
                                                         DmcVertexOut out, int flip,
                                                         unsigned long long* stats) {
  __shared__ uint64_t cc[256];
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour[c];
  __syncthreads();
  const int64_t n = g.ncells();
  for (int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cell < n;
       cell += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r = rec[cell];
    if (rec_nv(r) == 0) continue;
    int i, j, k;
    cell_ijk(g, cell, i, j, k);
    float u[8];
    load_corners(g, i, j, k, u);
    const unsigned cs = mc_case(u, g.iso_up);
    const uint64_t c = dmc_polygon(cs, u, g.iso, cc);
    const int ncnt = cnt_count(c);
    // bounding boxes of all contours (slice, cpp_dmc/DualMarchingCubes.cpp:114-136)
    CellBoxes bx;
    int flat = 0;
    for (int t = 0; t < ncnt; t++) {
      bx.b[t][0][0] = 1; bx.b[t][0][1] = 0;
      bx.b[t][1][0] = 1; bx.b[t][1][1] = 0;
      bx.b[t][2][0] = 1; bx.b[t][2][1] = 0;
      const int sz = cnt_size(c, t);
      for (int q = 0; q < sz; q++) {
        float ui[3];
        local_coord(cnt_edge(c, flat + q), u, g.iso, ui);
#pragma unroll
        for (int d = 0; d < 3; d++) {
          bx.b[t][d][0] = bx.b[t][d][0] > ui[d] ? ui[d] : bx.b[t][d][0];
          bx.b[t][d][1] = bx.b[t][d][1] < ui[d] ? ui[d] : bx.b[t][d][1];
        }
      }
      flat += sz;
    }
    int32_t vidx = voff[cell];
    flat = 0;
    for (int t = 0; t < ncnt; t++) {
      const int sz = cnt_size(c, t);
      bool used = false;
      for (int q = 0; q < sz; q++) used = used || edge_interior(g, i, j, k, cnt_edge(c, flat + q));
      if (used) {
        double p[3] = {0, 0, 0};
        for (int q = 0; q < sz; q++) {
          float ui[3];
          local_coord(cnt_edge(c, flat + q), u, g.iso, ui);
          p[0] += ui[0];
          p[1] += ui[1];
          p[2] += ui[2];
        }
        p[0] /= sz;
        p[1] /= sz;
        p[2] /= sz;
        representative_exact(u, g.iso, c, t, p, bx, stats);
        // normal: trilinear interpolation of the 8 corner gradients, normalised
        // (UniformGrid::normal, cpp_dmc/UniformGrid.h:286-298)
        double G[8][3];
#pragma unroll
        for (int q = 0; q < 8; q++) point_gradient(g, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1), G[q]);
        double nv[3];
        const double uu = p[0], vv = p[1], ww = p[2];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          double gq[8];
#pragma unroll
          for (int q = 0; q < 8; q++) gq[q] = flip ? G[q][d] * -1. : G[q][d];
          nv[d] = (1 - ww) * ((1 - vv) * ((1 - uu) * gq[0] + uu * gq[1]) + vv * ((1 - uu) * gq[2] + uu * gq[3])) +
                  ww * ((1 - vv) * ((1 - uu) * gq[4] + uu * gq[5]) + vv * ((1 - uu) * gq[6] + uu * gq[7]));
        }
        const double s_ = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
        nv[0] /= s_;
        nv[1] /= s_;
        nv[2] /= s_;
        // position (UniformGrid::position, cpp_dmc/UniformGrid.h:300-305)
        const double px = g.ox + (i + p[0]) * g.dx;
        const double py = g.oy + (j + p[1]) * g.dy;
        const double pz = g.oz + (k + p[2]) * g.dz;
        const int64_t o = 3 * (int64_t)vidx;
        out.v[o] = (float)px;
        out.v[o + 1] = (float)py;
        out.v[o + 2] = (float)pz;
        out.n[o] = (float)nv[0];
        out.n[o + 1] = (float)nv[1];
        out.n[o + 2] = (float)nv[2];
        if (out.v64) {
          out.v64[o] = px;
          out.v64[o + 1] = py;
          out.v64[o + 2] = pz;
        }
        if (out.vcell) {
          out.vcell[vidx] = cell;
          out.vuvw[o] = (float)p[0];
          out.vuvw[o + 1] = (float)p[1];
          out.vuvw[o + 2] = (float)p[2];
        }
        vidx++;
      }
      flat += sz;
    }
  }
}

// ------------------------------------------------------------------------------------------
// quads: the cell owning a crossed interior edge (its edge 0, 3 or 8) gathers the vertices of the
// four cells around it.  Slot by the side of the edge's first end vertex (get_vertex_pos,
// cpp_dmc/DualMarchingCubes.h:221-224); colour 3*parity(i,j,k) + axis (:177-180).
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) dmc_quad_kernel(Grid g, const uint32_t* rec, const int32_t* voff,
                                                       const int32_t* qoff, int32_t* quads, uint8_t* colors) {
  const int64_t n = g.ncells();
  // cell offsets (di, dj, dk) and local edge of the four cells around the owned edges 0, 3, 8
  // x edge: (0,-1,-1) e6, (0,0,-1) e4, (0,-1,0) e2, (0,0,0) e0
  // y edge: (-1,0,-1) e5, (0,0,-1) e7, (-1,0,0) e1, (0,0,0) e3
  // z edge: (-1,-1,0) e10, (0,-1,0) e11, (-1,0,0) e9, (0,0,0) e8
  const int AX_E[3] = {0, 3, 8};
  for (int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cell < n;
       cell += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r = rec[cell];
    if (rec_nq(r) == 0) continue;
    int i, j, k;
    cell_ijk(g, cell, i, j, k);
    const float f0 = g.at(i, j, k);
    const int neg = !(f0 >= g.iso_up);  // first end vertex below the isovalue
    const float fx = g.at(i + 1, j, k), fy = g.at(i, j + 1, k), fz = g.at(i, j, k + 1);
    const bool s0 = f0 >= g.iso_up;
    const bool crossed[3] = {s0 != (fx >= g.iso_up), s0 != (fy >= g.iso_up), s0 != (fz >= g.iso_up)};
    int32_t q = qoff[cell];
    const int par = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
    for (int a = 0; a < 3; a++) {
      if (!crossed[a] || !edge_interior(g, i, j, k, AX_E[a])) continue;
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
      for (int s = 0; s < 4; s++) {
        const int64_t nc = g.cell_index(i + di[s], j + dj[s], k + dk[s]);
        const uint32_t rn = rec[nc];
        qv[quad_slot(le[s], neg)] = voff[nc] + rec_rank(rn, le[s]);
      }
      reinterpret_cast<int4*>(quads)[q] = make_int4(qv[0], qv[1], qv[2], qv[3]);
      if (colors) colors[q] = (uint8_t)(3 * par + a);
      q++;
    }
  }
}

// ------------------------------------------------------------------------------------------
// host-side launches
// ------------------------------------------------------------------------------------------
int dmc_front_count(const Grid& g, DmcScratch& s, cudaStream_t st, Prof* prof) {
  const int64_t n = g.ncells();
  const int64_t tiles = ceil_div(n, kScanTile);
  {
    Stage t(prof, "dmc_classify", st);
    dmc_classify_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(g, s.rec, s.tile_sums, s.stats);
  }
  Stage t(prof, "dmc_scan", st);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(s.tile_sums, tiles, s.totals);
  dmc_offsets_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(n, s.rec, s.tile_sums, s.voff, s.qoff);
  return 3;
}

int64_t dmc_tiles(const Grid& g) { return ceil_div(g.ncells(), kScanTile); }

int dmc_front_emit(const Grid& g, DmcScratch& s, DmcVertexOut vo, int32_t* quads, uint8_t* colors, int flip,
                   int sms, cudaStream_t st, Prof* prof) {
  const int64_t n = g.ncells();
  const int64_t blocks = std::min<int64_t>(ceil_div(n, 128), (int64_t)sms * 16);
  {
    Stage t(prof, "dmc_vertex", st);
    dmc_vertex_kernel<<<(unsigned)blocks, 128, 0, st>>>(g, s.rec, s.voff, vo, flip, s.stats);
  }
  Stage t(prof, "dmc_quad", st);
  dmc_quad_kernel<<<(unsigned)blocks, 128, 0, st>>>(g, s.rec, s.voff, s.qoff, quads, colors);
  return 2;
}

}  // namespace tmc
