// Per-cell helpers of the DMC front end: corner loads, MC case, the per-cell record (used-contour
// count, owned quads, edge -> vertex rank map) shared by the extraction kernels and the
// static-scratch counting kernel.
#pragma once
#include "common.cuh"
#include "listing.cuh"

namespace tmc {

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

// Linear cell index -> (i, j, k); cell counts stay below 2^32 (checked by the runtime)
__device__ __forceinline__ void cell_ijk(const Grid& g, int64_t c, int& i, int& j, int& k) {
  const uint32_t cx = (uint32_t)(g.nx - 1), cy = (uint32_t)(g.ny - 1);
  const uint32_t cc = (uint32_t)c;  // cell indices of a volume stay below 2^32
  const uint32_t r = g.div_cx.div(cc);
  i = (int)(cc - r * cx);
  const uint32_t kk = g.div_cy.div(r);
  j = (int)(r - kk * cy);
  k = (int)kk;
}

// Record of a listed cell (case cs, neither 0 nor 255) from its contour word c (at most four
// contours); amb: the case is ambiguous (record bit 29).
__device__ __forceinline__ uint32_t record_from_contours(const Grid& g, int i, int j, int k, unsigned cs, uint64_t c,
                                                         bool amb) {
  const int ncnt = cnt_count(c);
  uint32_t rec = amb ? (1u << 29) : 0u;
  // a cell at least one cell away from every border has only interior edges (most listed cells)
  const bool inner = i >= 1 && j >= 1 && k >= 1 && i <= g.nx - 3 && j <= g.ny - 3 && k <= g.nz - 3;
  int nv = 0, flat = 0;
  for (int t = 0; t < ncnt; t++) {
    const int sz = cnt_size(c, t);
    bool used = inner;
    for (int q = 0; q < sz && !used; q++) used = edge_interior(g, i, j, k, cnt_edge(c, flat + q));
    if (used) {
      for (int q = 0; q < sz; q++) rec |= (uint32_t)nv << (5 + 2 * cnt_edge(c, flat + q));
      nv++;
    }
    flat += sz;
  }
  // owned quads: crossed interior edges 0 (x), 3 (y), 8 (z) at the cell's lower corner
  const uint32_t em = case_edge_mask(cs);
  int nq = 0;
  nq += ((em >> 0) & 1) && (inner || edge_interior(g, i, j, k, 0));
  nq += ((em >> 3) & 1) && (inner || edge_interior(g, i, j, k, 3));
  nq += ((em >> 8) & 1) && (inner || edge_interior(g, i, j, k, 8));
  rec |= (uint32_t)nv | ((uint32_t)nq << 3);
  return rec;
}

// Record of a listed cell; cc: the 256 packed case contours; u, the corners, are read only for the
// ambiguous cases (the decider).
__device__ __forceinline__ uint32_t classify_active(const Grid& g, int i, int j, int k, unsigned cs, const float* u,
                                                    const uint64_t* cc) {
  const bool amb = case_ambiguous(cs);
  const uint64_t c = amb ? dmc_polygon(cs, u, g.iso, cc) : table_contour(cc[cs]);
  return record_from_contours(g, i, j, k, cs, c, amb);
}

__device__ __forceinline__ uint32_t classify_cell(const Grid& g, int i, int j, int k, const uint64_t* cc,
                                                  unsigned long long* stats) {
  float u[8];
  load_corners(g, i, j, k, u);
  const unsigned cs = mc_case(u, g.iso_up);
  (void)stats;
  if (cs == 0 || cs == 255) return 0;
  return classify_active(g, i, j, k, cs, u, cc);
}

}  // namespace tmc
