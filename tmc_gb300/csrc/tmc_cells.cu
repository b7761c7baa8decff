// Topologically correct Marching Cubes (TMC) on the GPU, emitted in the reference's order.
//
// Order.  The reference CPU path t_mc (mc/MarchingCubes.cpp:151-317) walks cells in grid order
// and creates a vertex for a crossed edge the first time a cell touches it (std::map keyed by the
// global edge), in edge order 0..11, followed by the cell's inner vertices (p_slice,
// :323-1299); triangles are appended cell by cell.  The first cell touching an edge is the
// lowest-index cell around it, so each cell "owns" a fixed subset of its edges (those whose lower
// neighbours across the edge do not exist).  Hence
//   vertex index   = #vertices of earlier cells + rank among the cell's owned edges (or inner)
//   triangle index = #triangles of earlier cells + rank in the cell
// both exclusive prefix sums over cells; a triangle corner on an edge owned by a neighbour reads
// that neighbour's record.  No hash table, no atomics, deterministic output.
//
// Kernels:
//   tmc_classify_kernel  per-cell record: owned crossed edges, table triangle counts; ambiguous
//                        cells listed
//   tmc_amb_key/cursor/sort_kernel  the ambiguous list sorted by MC case
//   tmc_amb_count_kernel the ambiguous cells' p_slice (float64), once: counts into the cell records,
//                        triangles (local codes) and inner-vertex parameters into AmbRec records
//   tmc_offsets_kernel   in-tile scan -> per-cell vertex / triangle offsets
//   tmc_emit_kernel      edge vertices and table triangles
//   tmc_ambiguous_kernel the ambiguous cells' triangles and inner vertices from their records
#include "ffloat.cuh"
#include "listing.cuh"
#include "scan.cuh"
#include "tmc_cells.h"

namespace tmc {

__constant__ uint64_t c_tmc_tris[256] = TMC_TRIANGLES_INIT;

// per-cell record
//   bits 0-11  owned crossed edges
//   bits 12-14 inner vertices (0, 1 or 6)
//   bits 15-20 triangles
//   bit 21     ambiguous case
//   bit 22     a singular face the reference cannot triangulate (cell emits no triangle)
__device__ __forceinline__ uint32_t trec_owned(uint32_t r) { return r & 0xFFF; }
__device__ __forceinline__ int trec_inner(uint32_t r) { return (r >> 12) & 7; }
__device__ __forceinline__ int trec_ntri(uint32_t r) { return (r >> 15) & 63; }
__device__ __forceinline__ int trec_nv(uint32_t r) { return __popc(trec_owned(r)) + trec_inner(r); }

// cell counts stay below 2^32 (checked by the runtime), so 32-bit division suffices
__device__ __forceinline__ void tcell_ijk(const Grid& g, int64_t c, int& i, int& j, int& k) {
  const uint32_t cx = (uint32_t)(g.nx - 1), cy = (uint32_t)(g.ny - 1);
  const uint32_t cc = (uint32_t)c;  // cell indices of a volume stay below 2^32
  const uint32_t r = g.div_cx.div(cc);
  i = (int)(cc - r * cx);
  const uint32_t kk = g.div_cy.div(r);
  j = (int)(r - kk * cy);
  k = (int)kk;
}

__device__ __forceinline__ void tload_corners(const Grid& g, int i, int j, int k, float u[8]) {
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

// Edges a cell creates first: across the edge, along each other axis, the cell either sits on the
// far side of the edge (offset 1) or no lower neighbour exists (index 0).
__device__ __forceinline__ uint32_t owned_edges(int i, int j, int k) {
  uint32_t m = 0;
#pragma unroll
  for (int e = 0; e < 12; e++) {
    const int off = edge_off(e), ax = edge_axis(e);
    bool own = true;
    if (ax != 0) own = own && (((off >> 0) & 1) || i == 0);
    if (ax != 1) own = own && (((off >> 1) & 1) || j == 0);
    if (ax != 2) own = own && (((off >> 2) & 1) || k == 0);
    m |= (uint32_t)own << e;
  }
  return m;
}

// Owner cell of local edge e of cell (i,j,k) and the edge's local index there.
__device__ __forceinline__ void edge_owner(int i, int j, int k, int e, int& oi, int& oj, int& ok, int& oe) {
  const int off = edge_off(e), ax = edge_axis(e);
  const int gi = i + (off & 1), gj = j + ((off >> 1) & 1), gk = k + ((off >> 2) & 1);
  oi = (ax == 0) ? gi : (gi > 0 ? gi - 1 : 0);
  oj = (ax == 1) ? gj : (gj > 0 ? gj - 1 : 0);
  ok = (ax == 2) ? gk : (gk > 0 ? gk - 1 : 0);
  const int o = (gi - oi) | ((gj - oj) << 1) | ((gk - ok) << 2);  // offset of the edge in the owner
  // local edge with that offset and axis
#pragma unroll
  for (int q = 0; q < 12; q++)
    if (edge_axis(q) == ax && edge_off(q) == o) oe = q;
}

// ------------------------------------------------------------------------------------------
// cell geometry in float64 for the ambiguous path
// ------------------------------------------------------------------------------------------
// UGrid::gradient (mc/MarchingCubes.cpp:1451-1509): one-sided differences on the border
__device__ __forceinline__ void tmc_point_gradient(const Grid& g, int i, int j, int k, double out[3]) {
  if (i == 0) out[0] = ((double)g.at(i + 1, j, k) - (double)g.at(i, j, k)) / g.dx;
  else if (i == g.nx - 1) out[0] = ((double)g.at(i, j, k) - (double)g.at(i - 1, j, k)) / g.dx;
  else out[0] = ((double)g.at(i + 1, j, k) - (double)g.at(i - 1, j, k)) / (2 * g.dx);
  if (j == 0) out[1] = ((double)g.at(i, j + 1, k) - (double)g.at(i, j, k)) / g.dy;
  else if (j == g.ny - 1) out[1] = ((double)g.at(i, j, k) - (double)g.at(i, j - 1, k)) / g.dy;
  else out[1] = ((double)g.at(i, j + 1, k) - (double)g.at(i, j - 1, k)) / (2 * g.dy);
  if (k == 0) out[2] = ((double)g.at(i, j, k + 1) - (double)g.at(i, j, k)) / g.dz;
  else if (k == g.nz - 1) out[2] = ((double)g.at(i, j, k) - (double)g.at(i, j, k - 1)) / g.dz;
  else out[2] = ((double)g.at(i, j, k + 1) - (double)g.at(i, j, k - 1)) / (2 * g.dz);
}

__device__ __forceinline__ void cell_trilinear3(const double q[8][3], double u, double v, double w, double out[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++)
    out[d] = (1 - w) * ((1 - v) * (q[0][d] + u * (q[1][d] - q[0][d])) + v * (q[2][d] + u * (q[3][d] - q[2][d]))) +
             w * ((1 - v) * (q[4][d] + u * (q[5][d] - q[4][d])) + v * (q[6][d] + u * (q[7][d] - q[6][d])));
}

// The isovalue's parameter on crossed edge e (t_mc's edge coordinates, mc/MarchingCubes.cpp:241-254),
// float64.  p_slice reads them only on a singular face and in the tunnel / hexagon branch, so they
// are computed there, not for every ambiguous cell.
__device__ __forceinline__ double edge_coord(const double F[8], double iso, int e) {
  const int v0 = edge_v0(e), v1 = edge_v1(e);
  return (iso - F[v0]) / (F[v1] - F[v0]);
}

// e_vert (mc/MarchingCubes.cpp:902-911): local coordinate d of the point on edge e
__device__ __forceinline__ double e_vert(const double ecoord[12], int e, int d) {
  return (edge_axis(e) == d) ? ecoord[e] : (double)((edge_off(e) >> d) & 1);
}

// Triangles of p_slice: written out (3 vertex indices each), or, in the counting pass, kept as local
// vertex codes (0..11 the crossed edges, 12..17 the inner vertices; 5 bits each) in the cell's
// ambiguous-cell record, the first kAmbRecTris of them.  n counts them all.
constexpr int kAmbRecTris = 36;
struct TriSink {
  int32_t* out;     // 3 per triangle, or NULL
  uint16_t* codes;  // packed codes, or NULL
  int n;
  __device__ __forceinline__ void put(int a, int b, int c) {
    if (out) {
      out[3 * n] = a;
      out[3 * n + 1] = b;
      out[3 * n + 2] = c;
    } else if (codes && n < kAmbRecTris) {
      codes[n] = (uint16_t)(a | b << 5 | c << 10);
    }
    n++;
  }
};

// The record the counting pass keeps of an ambiguous cell, so that the emission pass does not run
// p_slice again (32 words, 16-byte aligned):
//   w[0]     slot of the cell
//   w[1]     bits 0-7 MC case, 8-13 triangles, 14-16 inner vertices, 17 triangles beyond the record
//            (emission runs p_slice again), 18 a singular face the reference cannot triangulate
//   w[2..13] six float64 parameters of the inner vertices: (u, v, w) of the single inner vertex, or
//            (u0, u1, v0, v1, w0, w1) of the six hexagon corners
//   w[14..31] kAmbRecTris triangles as packed local codes (TriSink)
constexpr int kAmbRecWords = 32;
struct __align__(16) AmbRec {
  uint32_t slot, info;
  double prm[6];
  uint16_t tri[kAmbRecTris];
};
static_assert(sizeof(AmbRec) == 4 * kAmbRecWords && kAmbRecWords == kTmcAmbRecWords, "ambiguous-cell record size");

struct AmbResult {
  int inner;     // inner vertices created
  bool error;    // singular face without a valid triangulation
};

// p_slice after the edge vertices (mc/MarchingCubes.cpp:418-1296), float64 throughout.
// vid[e]: global index of the vertex on crossed edge e; ibase: index of the first inner vertex.
// When `geo` is set, inner vertices are written there (positions/normals); when `prm` is set, the
// parameters they are made from (AmbRec::prm).
struct InnerOut {
  float* v;
  float* n;
  double* v64;
};

// Corners (u, v, w) of the inner hexagon (:831-840) from the quadratic's two roots per axis
__device__ __forceinline__ void hex_corners(const double ui[2], const double vi[2], const double wi[2],
                                            double hvt[6][3]) {
  const double c[6][3] = {{ui[0], vi[0], wi[0]}, {ui[0], vi[0], wi[1]}, {ui[1], vi[0], wi[1]},
                          {ui[1], vi[1], wi[1]}, {ui[1], vi[1], wi[0]}, {ui[0], vi[1], wi[0]}};
#pragma unroll
  for (int s = 0; s < 6; s++)
#pragma unroll
    for (int d = 0; d < 3; d++) hvt[s][d] = c[s][d];
}

// One inner vertex at local parameters (u, v, w): trilinear position and normal of the cell's corners,
// the normal normalised (the reference's arithmetic, :1073-1083 and :1283-1293).
__device__ __forceinline__ void inner_vertex(const double (*P)[3], const double (*N)[3], double u, double v, double w,
                                             const InnerOut& geo, int64_t index) {
  double ip[3], in[3];
  cell_trilinear3(P, u, v, w, ip);
  cell_trilinear3(N, u, v, w, in);
  const double factor = sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
  const int64_t o = 3 * index;
  for (int q = 0; q < 3; q++) {
    geo.v[o + q] = (float)ip[q];
    geo.n[o + q] = (float)(in[q] / factor);
    if (geo.v64) geo.v64[o + q] = ip[q];
  }
}

__device__ AmbResult p_slice_dev(unsigned ic, const double F[8], double iso, const int32_t vid[12], int32_t ibase,
                                 TriSink& tri, const double (*P)[3], const double (*N)[3], const InnerOut* geo,
                                 double* prm) {
  AmbResult res{0, false};
  uint64_t to = ~0ull;
  int f_flag = 0;
#pragma unroll 1
  for (int f = 0; f < 6; f++) {
    const uint32_t fv = face_v_pack(f), fe = face_e_pack(f);
    const double f0 = F[nib(fv, 0)], f1 = F[nib(fv, 1)], f2 = F[nib(fv, 2)], f3 = F[nib(fv, 3)];
    int fc = 0;
    if (f0 >= iso) fc |= 1;
    if (f1 >= iso) fc |= 2;
    if (f2 >= iso) fc |= 4;
    if (f3 >= iso) fc |= 8;
    int sep = 0;
    if (fc == 6 || fc == 9) {
      const double val = decider(f0, f1, f2, f3);
      if (val > iso) sep = 1;
      else if (val < iso) sep = 0;
      else {
        f_flag |= 1 << f;
        const unsigned e_flag = 0x218;
        // an ambiguous face: its four edges are crossed
        double ec0 = edge_coord(F, iso, nib(fe, 0)), ec1 = edge_coord(F, iso, nib(fe, 1)),
               ec2 = edge_coord(F, iso, nib(fe, 2)), ec3 = edge_coord(F, iso, nib(fe, 3));
        if ((e_flag >> (f * 2)) & 1) { ec0 = 1 - ec0; ec2 = 1 - ec2; }
        if ((e_flag >> (f * 2)) & 2) { ec1 = 1 - ec1; ec3 = 1 - ec3; }
        const bool c1 = (ec1 < ec3 && ec0 > ec2), c2 = (ec1 > ec3 && ec0 < ec2);
        if (!c1 && !c2) {
          res.error = true;
          return res;
        }
        sep = (fc == 6) ? (c1 ? 0 : 1) : (c1 ? 1 : 0);
      }
    }
    face_segments(fc, sep, fe, to);
  }
  const uint64_t c = connect_contours(to, case_edge_mask(ic));
  const int cnt = cnt_count(c);

  // inner-ambiguity quadratic (:715-795)
  double ui[2] = {0, 0}, vi[2] = {0, 0}, wi[2] = {0, 0};
  unsigned q_sol = 0;
  const double a = (F[0] - F[1]) * (-F[6] + F[7] + F[4] - F[5]) - (F[4] - F[5]) * (-F[2] + F[3] + F[0] - F[1]);
  const double b = (iso - F[0]) * (-F[6] + F[7] + F[4] - F[5]) + (F[0] - F[1]) * (F[6] - F[4]) -
                   (iso - F[4]) * (-F[2] + F[3] + F[0] - F[1]) - (F[4] - F[5]) * (F[2] - F[0]);
  const double cc = (iso - F[0]) * (F[6] - F[4]) - (iso - F[4]) * (F[2] - F[0]);
  double d = b * b - 4 * a * cc;
  if (d > 0) {
    d = sqrt(d);
    ui[0] = (-b - d) / (2 * a);
    ui[1] = (-b + d) / (2 * a);
    double g1 = F[0] * (1 - ui[0]) + F[1] * ui[0];
    double g2 = F[2] * (1 - ui[0]) + F[3] * ui[0];
    vi[0] = (iso - g1) / (g2 - g1);
    if (isnan(vi[0]) || isinf(vi[0])) vi[0] = -1.f;
    g1 = F[0] * (1 - ui[1]) + F[1] * ui[1];
    g2 = F[2] * (1 - ui[1]) + F[3] * ui[1];
    vi[1] = (iso - g1) / (g2 - g1);
    if (isnan(vi[1]) || isinf(vi[1])) vi[1] = -1.f;
    g1 = F[0] * (1 - ui[0]) + F[1] * ui[0];
    g2 = F[4] * (1 - ui[0]) + F[5] * ui[0];
    wi[0] = (iso - g1) / (g2 - g1);
    if (isnan(wi[0]) || isinf(wi[0])) wi[0] = -1.f;
    g1 = F[0] * (1 - ui[1]) + F[1] * ui[1];
    g2 = F[4] * (1 - ui[1]) + F[5] * ui[1];
    wi[1] = (iso - g1) / (g2 - g1);
    if (isnan(wi[1]) || isinf(wi[1])) wi[1] = -1.f;
    if (f_flag & 1) { if (wi[0] < wi[1]) wi[0] = 0; else wi[1] = 0; }
    if (f_flag & 2) { if (wi[0] > wi[1]) wi[1] = 1; else wi[1] = 1; }
    if (f_flag & 4) { if (vi[0] < vi[1]) vi[0] = 0; else vi[1] = 0; }
    if (f_flag & 8) { if (vi[0] > vi[1]) vi[0] = 1; else vi[1] = 1; }
    if (f_flag & 16) { if (ui[0] < ui[1]) ui[0] = 0; else ui[1] = 0; }
    if (f_flag & 32) { if (ui[0] > ui[1]) ui[0] = 1; else ui[1] = 1; }
    if (0 < ui[0] && ui[0] < 1) q_sol |= 1;
    if (0 < ui[1] && ui[1] < 1) q_sol |= 2;
    if (0 < vi[0] && vi[0] < 1) q_sol |= 4;
    if (0 < vi[1] && vi[1] < 1) q_sol |= 8;
    if (0 < wi[0] && wi[0] < 1) q_sol |= 16;
    if (0 < wi[1] && wi[1] < 1) q_sol |= 32;
  }

  if (__popc(q_sol) == 6) {
    // tunnel or 12-vertex contour: inner hexagon (:831-1083)
    double ecoord[12];
    const uint32_t emask = case_edge_mask(ic);
    for (int e = 0; e < 12; e++) ecoord[e] = (emask >> e) & 1 ? edge_coord(F, iso, e) : 0.0;
    double hvt[6][3];
    hex_corners(ui, vi, wi, hvt);
    int not_tunnel = 0xF;
    if (cnt == 3) {
      const double uc_min = (ui[0] < ui[1]) ? ui[0] : ui[1];
      const double uc_max = (ui[0] < ui[1]) ? ui[1] : ui[0];
      int flat = 0;
      for (int t = 0; t < cnt; t++) {
        const int sz = cnt_size(c, t);
        if (sz == 3) {
          double umin = 2, umax = -2;
          const int e0 = cnt_edge(c, flat), e1 = cnt_edge(c, flat + 1), e2 = cnt_edge(c, flat + 2);
          const double u_e0 = e_vert(ecoord, e0, 0), u_e1 = e_vert(ecoord, e1, 0), u_e2 = e_vert(ecoord, e2, 0);
          umin = (u_e0 < umin) ? u_e0 : umin;
          umin = (u_e1 < umin) ? u_e1 : umin;
          umin = (u_e2 < umin) ? u_e2 : umin;
          umax = (u_e0 > umax) ? u_e0 : umax;
          umax = (u_e1 > umax) ? u_e1 : umax;
          umax = (u_e2 > umax) ? u_e1 : umax;  // the reference keeps u_e1 here
          if (uc_min > umax || uc_max < umin) {
            not_tunnel = t;
            tri.put(vid[e0], vid[e1], vid[e2]);
          }
        }
        flat += sz;
      }
    }
    if (geo)
      for (int s = 0; s < 6; s++) inner_vertex(P, N, hvt[s][0], hvt[s][1], hvt[s][2], *geo, (int64_t)ibase + s);
    if (prm) {
      prm[0] = ui[0]; prm[1] = ui[1]; prm[2] = vi[0]; prm[3] = vi[1]; prm[4] = wi[0]; prm[5] = wi[1];
    }
    res.inner = 6;
    unsigned char tcon[12];
    int flat = 0;
    for (int t = 0; t < cnt; t++) {
      const int sz = cnt_size(c, t);
      if (not_tunnel != t) {
        for (int r = 0; r < sz; r++) {
          unsigned idx = (unsigned)-1;
          double dist = 1000.;
          const int ci = cnt_edge(c, flat + r);
          const double ue = e_vert(ecoord, ci, 0), ve = e_vert(ecoord, ci, 1), we = e_vert(ecoord, ci, 2);
          for (int s = 0; s < 6; s++) {
            const double uval = ue - hvt[s][0], vval = ve - hvt[s][1], wval = we - hvt[s][2];
            const double val = uval * uval + vval * vval + wval * wval;
            if (dist > val) {
              idx = (unsigned)s;
              dist = val;
            }
          }
          tcon[ci] = (unsigned char)idx;
        }
        for (int r = 0; r < sz; r++) {
          const int tid1 = cnt_edge(c, flat + r), tid2 = cnt_edge(c, flat + (r + 1) % sz);
          const int cid1 = tcon[tid1], cid2 = tcon[tid2];
          const int rr = (cid1 - cid2) < 0 ? cid2 - cid1 : cid1 - cid2;
          const int dst = rr > 2 ? 6 - rr : rr;
          if (dst == 0) {
            tri.put(vid[tid1], vid[tid2], ibase + cid1);
          } else if (dst == 1) {
            double l1 = 0, l2 = 0;
            {
              const double a0 = e_vert(ecoord, tid1, 0) - hvt[cid2][0], a1 = e_vert(ecoord, tid1, 1) - hvt[cid2][1],
                           a2 = e_vert(ecoord, tid1, 2) - hvt[cid2][2];
              l1 = a0 * a0 + a1 * a1 + a2 * a2;
              const double b0 = e_vert(ecoord, tid2, 0) - hvt[cid1][0], b1 = e_vert(ecoord, tid2, 1) - hvt[cid1][1],
                           b2 = e_vert(ecoord, tid2, 2) - hvt[cid1][2];
              l2 = b0 * b0 + b1 * b1 + b2 * b2;
            }
            if (l1 < l2) {
              tri.put(vid[tid1], vid[tid2], ibase + cid2);
              tri.put(vid[tid1], ibase + cid2, ibase + cid1);
            } else {
              tri.put(vid[tid1], vid[tid2], ibase + cid1);
              tri.put(vid[tid2], ibase + cid2, ibase + cid1);
            }
          } else if (dst == 2) {
            const int dmax = (cid1 > cid2) ? cid1 : cid2, dmin = (cid1 < cid2) ? cid1 : cid2;
            const int cidm = ((dmax + 2) % 6 == dmin) ? (dmax + 1) % 6 : (dmax + dmin) / 2;
            tri.put(vid[tid1], vid[tid2], ibase + cidm);
            tri.put(vid[tid1], ibase + cidm, ibase + cid1);
            tri.put(vid[tid2], ibase + cid2, ibase + cidm);
          }
        }
      }
      flat += sz;
    }
    if (cnt == 1) {
      const bool s_ = decider(F[0], F[1], F[2], F[3]) <= iso;
      const bool of_ = (wi[1] < wi[0]) ? s_ : !s_;
      const int t0 = ibase, t1 = ibase + 1, t2 = ibase + 2, t3 = ibase + 3, t4 = ibase + 4, t5 = ibase + 5;
      if (!of_) {
        tri.put(t0, t2, t1); tri.put(t2, t4, t3); tri.put(t0, t5, t4); tri.put(t0, t4, t2);
      } else {
        tri.put(t0, t1, t2); tri.put(t2, t3, t4); tri.put(t0, t4, t5); tri.put(t0, t2, t4);
      }
    }
    return res;
  }
  // no tunnel
  const unsigned nr_u = ((q_sol & 0x5) == 0x5) + ((q_sol & 0xA) == 0xA);
  const unsigned nr_v = ((q_sol & 0x11) == 0x11) + ((q_sol & 0x22) == 0x22);
  const unsigned nr_w = ((q_sol & 0x18) == 0x18) + ((q_sol & 0x24) == 0x24);
  const unsigned nr_t = nr_u + nr_v + nr_w;
  if (nr_t == nr_u || nr_t == nr_v || nr_t == nr_w) {
    int flat = 0;
    for (int t = 0; t < cnt; t++) {
      const int sz = cnt_size(c, t);
      int e[6];
      for (int q = 0; q < 6; q++) e[q] = (q < sz) ? vid[cnt_edge(c, flat + q)] : -1;
      switch (sz) {
        case 3: tri.put(e[0], e[1], e[2]); break;
        case 4: tri.put(e[0], e[1], e[2]); tri.put(e[0], e[2], e[3]); break;
        case 5: tri.put(e[0], e[1], e[2]); tri.put(e[0], e[2], e[3]); tri.put(e[0], e[3], e[4]); break;
        case 6:
          tri.put(e[0], e[1], e[3]); tri.put(e[1], e[2], e[3]); tri.put(e[0], e[3], e[4]); tri.put(e[0], e[4], e[5]);
          break;
        default: break;
      }
      flat += sz;
    }
    return res;
  }
  // saddle points: one inner vertex (:1178-1296)
  const unsigned fs00 = q_sol & 1, fs01 = (q_sol >> 1) & 1, fs10 = (q_sol >> 2) & 1, fs11 = (q_sol >> 3) & 1,
                 fs20 = (q_sol >> 4) & 1, fs21 = (q_sol >> 5) & 1;
  const unsigned fc1 = fs00 * fs10 + fs01 * fs11;
  const unsigned fc2 = fs00 * fs20 + fs01 * fs21;
  const unsigned fc3 = fs10 * fs21 + fs11 * fs20;
  const unsigned c_faces = fc1 + fc2 + fc3;
  double uc = 0, vc = 0, wc = 0;
  if (c_faces == 2) {
    if (fc1 == 0) {
      uc = fs00 * ui[0] + fs01 * ui[1]; vc = fs10 * vi[0] + fs11 * vi[1]; wc = fs10 * wi[1] + fs11 * wi[0];
    } else if (fc2 == 0) {
      uc = fs00 * ui[0] + fs01 * ui[1]; vc = fs00 * vi[0] + fs01 * vi[1]; wc = fs00 * wi[1] + fs01 * wi[0];
    } else if (fc3 == 0) {
      uc = fs10 * ui[0] + fs11 * ui[1]; vc = fs10 * vi[0] + fs11 * vi[1]; wc = fs10 * wi[0] + fs11 * wi[1];
    }
  } else if (c_faces == 3) {
    uc = (fs00 * ui[0] + fs01 * ui[1]) / (int)(fs00 + fs01);
    vc = (fs10 * vi[0] + fs11 * vi[1]) / (int)(fs10 + fs11);
    wc = (fs20 * wi[0] + fs21 * wi[1]) / (int)(fs20 + fs21);
  } else if (c_faces == 4) {
    const unsigned nu = fs00 + fs01, nv = fs10 + fs11, nw = fs20 + fs21;
    if (nw == 1) {
      uc = fs20 * ui[0] + fs21 * ui[1]; vc = fs21 * vi[0] + fs20 * vi[1]; wc = fs20 * wi[0] + fs21 * wi[1];
    } else if (nv == 1) {
      uc = fs10 * ui[0] + fs11 * ui[1]; vc = fs10 * vi[0] + fs11 * vi[1]; wc = fs11 * wi[0] + fs10 * wi[1];
    } else if (nu == 1) {
      uc = fs00 * ui[0] + fs01 * ui[1]; vc = fs00 * vi[0] + fs01 * vi[1]; wc = fs00 * wi[0] + fs01 * wi[1];
    }
  }
  bool pt_used = false;
  int flat = 0;
  for (int t = 0; t < cnt; t++) {
    const int sz = cnt_size(c, t);
    if (sz == 3) {
      tri.put(vid[cnt_edge(c, flat)], vid[cnt_edge(c, flat + 1)], vid[cnt_edge(c, flat + 2)]);
    } else {
      pt_used = true;
      for (int r = 0; r < sz; r++) tri.put(vid[cnt_edge(c, flat + r)], vid[cnt_edge(c, flat + (r + 1) % sz)], ibase);
    }
    flat += sz;
  }
  if (pt_used) {
    res.inner = 1;
    if (geo) inner_vertex(P, N, uc, vc, wc, *geo, ibase);
    if (prm) {
      prm[0] = uc; prm[1] = vc; prm[2] = wc;
    }
  }
  return res;
}

// corner data of an ambiguous cell in float64: values, positions, normals
struct AmbCell {
  double F[8];
  double P[8][3];
  double N[8][3];
};

// corner positions and gradients (the inner vertices' trilinear sources)
__device__ __forceinline__ void amb_geometry(const Grid& g, int i, int j, int k, double P[8][3], double N[8][3]) {
  for (int q = 0; q < 8; q++) {
    const int ii = i + (q & 1), jj = j + ((q >> 1) & 1), kk = k + ((q >> 2) & 1);
    P[q][0] = g.ox + ii * g.dx;
    P[q][1] = g.oy + jj * g.dy;
    P[q][2] = g.oz + kk * g.dz;
    tmc_point_gradient(g, ii, jj, kk, N[q]);
  }
}

// Corner positions alone (float64, as amb_geometry).
__device__ __forceinline__ void amb_positions(const Grid& g, int i, int j, int k, double P[8][3]) {
  const double x[2] = {g.ox + i * g.dx, g.ox + (i + 1) * g.dx};
  const double y[2] = {g.oy + j * g.dy, g.oy + (j + 1) * g.dy};
  const double z[2] = {g.oz + k * g.dz, g.oz + (k + 1) * g.dz};
#pragma unroll
  for (int q = 0; q < 8; q++) {
    P[q][0] = x[q & 1];
    P[q][1] = y[(q >> 1) & 1];
    P[q][2] = z[(q >> 2) & 1];
  }
}

// tmc_point_gradient in float-float: the exact float difference times 1/(2 spacing) (1/spacing on
// the border), within ~2^-46 of the reference's float64 quotient.
__device__ __forceinline__ ffx::ff grad_axis_ff(float hi_v, float lo_v, bool border, float s_hi, float s_lo) {
  const float m = border ? 2.0f : 1.0f;  // 1/spacing = 2 * 1/(2 spacing), exactly
  return ffx::ff_mul(ffx::two_sum(hi_v, -lo_v), ffx::ff{s_hi * m, s_lo * m});
}
__device__ __forceinline__ void tmc_gradient_ff(const Grid& g, int i, int j, int k, ffx::ff out[3]) {
  const int i1 = i == g.nx - 1 ? i : i + 1, i0 = i == 0 ? 0 : i - 1;
  const int j1 = j == g.ny - 1 ? j : j + 1, j0 = j == 0 ? 0 : j - 1;
  const int k1 = k == g.nz - 1 ? k : k + 1, k0 = k == 0 ? 0 : k - 1;
  out[0] = grad_axis_ff(g.at(i1, j, k), g.at(i0, j, k), i == 0 || i == g.nx - 1, g.inv2_hi[0], g.inv2_lo[0]);
  out[1] = grad_axis_ff(g.at(i, j1, k), g.at(i, j0, k), j == 0 || j == g.ny - 1, g.inv2_hi[1], g.inv2_lo[1]);
  out[2] = grad_axis_ff(g.at(i, j, k1), g.at(i, j, k0), k == 0 || k == g.nz - 1, g.inv2_hi[2], g.inv2_lo[2]);
}

// a + t (b - a), all float pairs
__device__ __forceinline__ ffx::ff ff_lerp_ff(ffx::ff a, ffx::ff b, ffx::ff t) {
  return ffx::ff_add(a, ffx::ff_mul(ffx::ff_sub(b, a), t));
}

// One inner vertex of the emission pass: the float64 position as inner_vertex forms it, the normal
// from the float-float corner gradients N (trilinear at (u, v, w), normalised; within a few 2^-40 of
// the reference's float64 normal).  Only the float32 rounding of the normal is output, so the float
// pairs serve wherever the gradients do not cancel to below 2^-10 of their size; there it returns
// false and the caller computes the normal in float64.
__device__ __forceinline__ bool inner_vertex_ff(const double (*P)[3], const ffx::ff (*N)[3], float scale, double u,
                                                double v, double w, const InnerOut& geo, int64_t index) {
  double ip[3];
  cell_trilinear3(P, u, v, w, ip);
  const ffx::ff U = ffx::ff_from_double(u), V = ffx::ff_from_double(v), W = ffx::ff_from_double(w);
  ffx::ff in[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const ffx::ff a0 = ff_lerp_ff(N[0][d], N[1][d], U), a1 = ff_lerp_ff(N[2][d], N[3][d], U);
    const ffx::ff a2 = ff_lerp_ff(N[4][d], N[5][d], U), a3 = ff_lerp_ff(N[6][d], N[7][d], U);
    in[d] = ff_lerp_ff(ff_lerp_ff(a0, a1, V), ff_lerp_ff(a2, a3, V), W);
  }
  const ffx::ff dot =
      ffx::ff_add(ffx::ff_add(ffx::ff_mul(in[0], in[0]), ffx::ff_mul(in[1], in[1])), ffx::ff_mul(in[2], in[2]));
  if (!(dot.hi > 0.0f) || !(scale <= 0x1p10f * sqrtf(dot.hi))) return false;
  // 1/sqrt(dot): float estimate and one Newton step in float-float
  const float r0 = rsqrtf(dot.hi);
  const ffx::ff h = ffx::ff_mul_f(ffx::ff_mul_f(dot, r0), r0);
  const ffx::ff r = ffx::ff_mul_f(ffx::ff_sub(ffx::ff_from(1.5f), ffx::ff_mul_f(h, 0.5f)), r0);
  const int64_t o = 3 * index;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    geo.v[o + q] = (float)ip[q];
    geo.n[o + q] = ffx::ff_mul(in[q], r).hi;
    if (geo.v64) geo.v64[o + q] = ip[q];
  }
  return true;
}

__device__ void load_amb_cell(const Grid& g, int i, int j, int k, const float u[8], AmbCell& a, bool geometry) {
#pragma unroll
  for (int q = 0; q < 8; q++) a.F[q] = u[q];
  if (geometry) amb_geometry(g, i, j, k, a.P, a.N);
}

// ------------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------------
// One block per kScanTile consecutive cells.  Pass 1: MC cases from the warp-ballot corner rows
// (warp_cases) and the listing of the crossed cells in cell order (list_tile).  Pass 2: the records
// of the listed cells at their slots (owned crossed edges, table triangle counts); ambiguous cells are
// listed by slot (amb_list, warp-aggregated appends) for the float64 counting pass.
template <bool kGen>
__global__ void __launch_bounds__(kScanThreads, 6) tmc_classify_kernel(CellSpace space, int64_t tile0, uint32_t* rec,
                                                                   uint16_t* cellof, CellMask* mask,
                                                                   unsigned long long* tile_sums,
                                                                   unsigned long long* stats, uint32_t* amb_list,
                                                                   unsigned* amb_n) {
  const int64_t tile = tile0 + blockIdx.x;
  __shared__ uint16_t act_list[kScanTile];
  __shared__ uint8_t case_of[kScanTile];
  __shared__ uint32_t wmask[kScanTile / 32], wpre[kScanTile / 32];
  __shared__ int total;
  __shared__ unsigned long long tile_sum;
  if (threadIdx.x == 0) tile_sum = 0;
  const Grid g = space.grid_of_tile(tile);
  const int64_t n = g.ncells();
  const int64_t vbase = tile * kScanTile;
  const int lane = threadIdx.x & 31;
  const unsigned actbits = tile_cases<kGen>(g, space.n, vbase, case_of);
  const int na = list_tile(actbits, tile, mask, wmask, wpre, act_list, &total);
  unsigned long long local = 0, amb = 0;
  for (int a = threadIdx.x; a < na; a += blockDim.x) {
    const int off = act_list[a];
    const uint32_t slot = (uint32_t)(vbase + a);
    int i, j, k;
    tcell_ijk(g, vbase + off - g.vbase, i, j, k);
    const unsigned cs = case_of[off];
    // away from the lower borders a cell owns a fixed set of edges (folded at compile time)
    uint32_t r = case_edge_mask(cs) & ((i > 0 && j > 0 && k > 0) ? owned_edges(1, 1, 1) : owned_edges(i, j, k));
    const bool listed = case_ambiguous(cs);
    // ambiguous: counted by tmc_amb_count_kernel (float64), which adds to this tile's sums
    r |= listed ? (1u << 21) : (uint32_t)(c_tmc_tris[cs] & 0xF) << 15;
    amb += listed;
    rec[slot] = r;
    cellof[slot] = (uint16_t)off;
    local += ((unsigned long long)trec_nv(r) << 32) | (unsigned long long)trec_ntri(r);
    const unsigned am = __activemask();
    const unsigned bal = __ballot_sync(am, listed);
    if (bal) {
      const int leader = __ffs(bal) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(amb_n, (unsigned)__popc(bal));
      base = __shfl_sync(am, base, leader);
      if (listed) amb_list[base + __popc(bal & ((1u << lane) - 1u))] = slot;
    }
  }
  for (int o = 16; o; o >>= 1) {
    local += __shfl_down_sync(0xffffffffu, local, o);
    amb += __shfl_down_sync(0xffffffffu, amb, o);
  }
  if (lane == 0 && local) atomicAdd(&tile_sum, local);
  if (lane == 0 && amb) atomicAdd(stats + 1, amb);
  if (threadIdx.x == 0 && na) atomicAdd(stats + 0, (unsigned long long)na);
  __syncthreads();
  if (threadIdx.x == 0) tile_sums[tile] = tile_sum;
}

// The classification lists the ambiguous cells in no useful order; p_slice's branches follow the MC
// case, so the list is sorted by case (counting sort over the 256 cases) before the float64 passes:
// the lanes of a warp then mostly take the same branches (the float64 pipe issues for the whole warp
// whatever its active lanes).  Key pass: each cell's case and the per-case counts.
__global__ void __launch_bounds__(256) tmc_amb_key_kernel(CellSpace space, const uint16_t* cellof, const uint32_t* list,
                                                          int64_t n, uint8_t* key, unsigned* hist) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t vcell = slot_cell(cellof, list[a]);
    const Grid g = space.grid_of_tile(vcell / kScanTile);
    int i, j, k;
    tcell_ijk(g, vcell - g.vbase, i, j, k);
    float u[8];
    tload_corners(g, i, j, k, u);
    unsigned cs = 0;
#pragma unroll
    for (int v = 0; v < 8; v++) cs |= (unsigned)(u[v] >= g.iso_up) << v;
    key[a] = (uint8_t)cs;
    atomicAdd(&h[cs], 1u);
  }
  __syncthreads();
  if (h[threadIdx.x]) atomicAdd(hist + threadIdx.x, h[threadIdx.x]);
}

// exclusive scan of the 256 counts into the scatter cursors (one block of 256 threads)
__global__ void tmc_amb_cursor_kernel(const unsigned* hist, unsigned* cursor) {
  __shared__ unsigned x[256];
  x[threadIdx.x] = hist[threadIdx.x];
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const unsigned y = threadIdx.x >= (unsigned)o ? x[threadIdx.x - o] : 0u;
    __syncthreads();
    x[threadIdx.x] += y;
    __syncthreads();
  }
  cursor[threadIdx.x] = x[threadIdx.x] - hist[threadIdx.x];
}

__global__ void tmc_amb_sort_kernel(const uint32_t* list, const uint8_t* key, int64_t n, unsigned* cursor,
                                    uint32_t* sorted) {
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
    sorted[atomicAdd(cursor + key[a], 1u)] = list[a];
}

// Ambiguous cells from the classification's list: p_slice in counting mode (float64); the counts go
// into the cell record and, atomically, into the cell's tile sum (one thread per listed cell, no
// tile barrier to wait on).  The triangles (as local codes) and the inner vertices' parameters go
// into the cell's ambiguous-cell record, which the emission pass reads instead of running p_slice.
__global__ void __launch_bounds__(128) tmc_amb_count_kernel(CellSpace space, const uint16_t* cellof, uint32_t* rec,
                                                            unsigned long long* tile_sums,
                                                            unsigned long long* stats, const uint32_t* list,
                                                            const unsigned* count, AmbRec* recs) {
  const unsigned na = *count;
  unsigned long long sing = 0;
  for (unsigned a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) {
    const uint32_t slot = list[a];
    const int64_t vcell = slot_cell(cellof, slot);
    const Grid g = space.grid_of_tile(vcell / kScanTile);
    const int64_t cell = vcell - g.vbase;
    int i, j, k;
    tcell_ijk(g, cell, i, j, k);
    float u[8];
    tload_corners(g, i, j, k, u);
    unsigned cs = 0;
#pragma unroll
    for (int v = 0; v < 8; v++) cs |= (unsigned)(u[v] >= g.iso_up) << v;
    AmbCell amb;
    load_amb_cell(g, i, j, k, u, amb, false);
    int32_t vid[12];
    for (int e = 0; e < 12; e++) vid[e] = e;  // local codes: edges 0..11, inner vertices from 12
    AmbRec& R = recs[a];
    TriSink ts{nullptr, R.tri, 0};
    const AmbResult ar = p_slice_dev(cs, amb.F, g.iso, vid, 12, ts, amb.P, amb.N, nullptr, R.prm);
    R.slot = slot;
    R.info = cs | (uint32_t)ts.n << 8 | (uint32_t)ar.inner << 14 | (ts.n > kAmbRecTris ? (1u << 17) : 0u) |
             (ar.error ? (1u << 18) : 0u);
    rec[slot] |= (uint32_t)ar.inner << 12 | (uint32_t)ts.n << 15 | (ar.error ? (1u << 22) : 0u);
    const unsigned long long add = ((unsigned long long)ar.inner << 32) | (unsigned long long)ts.n;
    if (add) atomicAdd(tile_sums + (slot >> kTileShift), add);
    sing += ar.error;
  }
  if (sing) atomicAdd(stats + 5, sing);
}

// In-tile exclusive scan of the listed cells' records -> their vertex and triangle offsets (blocked
// layout over the tile's slots).
__global__ void __launch_bounds__(32 * kOffsetWarps) tmc_offsets_kernel(const CellMask* mask, const uint32_t* rec,
                                                                       const unsigned long long* tile_off,
                                                                       int64_t tiles, int32_t* voff, int32_t* toff) {
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
    for (int s = 0; s < kScanItems; s++) sum += ((unsigned long long)trec_nv(r[s]) << 32) | trec_ntri(r[s]);
    const unsigned long long inc = warp_inclusive_scan(sum);
    unsigned long long pre = carry + inc - sum;
    carry += __shfl_sync(0xffffffffu, inc, 31);
    int32_t vo[kScanItems], to[kScanItems];
#pragma unroll
    for (int s = 0; s < kScanItems; s++) {
      vo[s] = (int32_t)(pre >> 32);
      to[s] = (int32_t)(pre & 0xffffffffull);
      pre += ((unsigned long long)trec_nv(r[s]) << 32) | trec_ntri(r[s]);
    }
    store8(voff, first, end, vo);
    store8(toff, first, end, to);
  }
}

// corner value v of a cell's eight (selects, so that a run-time index keeps u in registers)
__device__ __forceinline__ float pick8(const float u[8], int v) {
  float r = u[0];
#pragma unroll
  for (int q = 1; q < 8; q++) r = (v == q) ? u[q] : r;
  return r;
}

// edge vertex: interpolation as t_mc (mc/MarchingCubes.cpp:241-254), float64
__device__ __forceinline__ void edge_vertex_f64(const Grid& g, int i, int j, int k, int e, const float u[8],
                                                const TmcVertexOut& out, int32_t idx) {
  const int v0 = edge_v0(e), v1 = edge_v1(e);
  const double F0 = pick8(u, v0), F1 = pick8(u, v1);
  const double l = (g.iso - F0) / (F1 - F0);
  const int i0 = i + (v0 & 1), j0 = j + ((v0 >> 1) & 1), k0 = k + ((v0 >> 2) & 1);
  const int i1 = i + (v1 & 1), j1 = j + ((v1 >> 1) & 1), k1 = k + ((v1 >> 2) & 1);
  const double p0[3] = {g.ox + i0 * g.dx, g.oy + j0 * g.dy, g.oz + k0 * g.dz};
  const double p1[3] = {g.ox + i1 * g.dx, g.oy + j1 * g.dy, g.oz + k1 * g.dz};
  double n0[3], n1[3];
  tmc_point_gradient(g, i0, j0, k0, n0);
  tmc_point_gradient(g, i1, j1, k1, n1);
  double ip[3], in[3];
#pragma unroll
  for (int d = 0; d < 3; d++) ip[d] = (1 - l) * p0[d] + l * p1[d];
#pragma unroll
  for (int d = 0; d < 3; d++) in[d] = (1 - l) * n0[d] + l * n1[d];
  const double nl = sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
  const int64_t o = 3 * (int64_t)idx;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    out.v[o + d] = (float)ip[d];
    out.n[o + d] = (float)(in[d] / nl);
    if (out.v64) out.v64[o + d] = ip[d];
  }
}

// edge vertex in float32 (positions within an ulp: the grid coordinate i + l is formed exactly as a
// float pair); the float64 variant above is used when float64 positions are requested
__device__ __forceinline__ void tmc_gradient_f(const Grid& g, int i, int j, int k, const float inv[3],
                                               const float inv2[3], float out[3]) {
  if (i == 0) out[0] = (g.at(i + 1, j, k) - g.at(i, j, k)) * inv[0];
  else if (i == g.nx - 1) out[0] = (g.at(i, j, k) - g.at(i - 1, j, k)) * inv[0];
  else out[0] = (g.at(i + 1, j, k) - g.at(i - 1, j, k)) * inv2[0];
  if (j == 0) out[1] = (g.at(i, j + 1, k) - g.at(i, j, k)) * inv[1];
  else if (j == g.ny - 1) out[1] = (g.at(i, j, k) - g.at(i, j - 1, k)) * inv[1];
  else out[1] = (g.at(i, j + 1, k) - g.at(i, j - 1, k)) * inv2[1];
  if (k == 0) out[2] = (g.at(i, j, k + 1) - g.at(i, j, k)) * inv[2];
  else if (k == g.nz - 1) out[2] = (g.at(i, j, k) - g.at(i, j, k - 1)) * inv[2];
  else out[2] = (g.at(i, j, k + 1) - g.at(i, j, k - 1)) * inv2[2];
}

__device__ __forceinline__ void edge_vertex_f32(const Grid& g, int i, int j, int k, int e, const float u[8],
                                                const TmcVertexOut& out, int32_t idx, const float inv[3],
                                                const float inv2[3]) {
  const int v0 = edge_v0(e), v1 = edge_v1(e), ax = edge_axis(e);
  const float F0 = pick8(u, v0), F1 = pick8(u, v1);
  const float l = (g.iso_f - F0) / (F1 - F0);
  const int i0 = i + (v0 & 1), j0 = j + ((v0 >> 1) & 1), k0 = k + ((v0 >> 2) & 1);
  const int i1 = i + (v1 & 1), j1 = j + ((v1 >> 1) & 1), k1 = k + ((v1 >> 2) & 1);
  const int gi[3] = {i0, j0, k0};
  const int64_t base = 3 * (int64_t)idx;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    // origin + (index + l) * spacing, with index + l exact as a float pair
    const ffx::ff t = (d == ax) ? ffx::two_sum((float)gi[d], l) : ffx::ff_from((float)gi[d]);
    const ffx::ff x = ffx::ff_add(ffx::ff{g.org_hi[d], g.org_lo[d]}, ffx::ff_mul(t, ffx::ff{g.sp_hi[d], g.sp_lo[d]}));
    out.v[base + d] = x.hi + x.lo;
  }
  float n0[3], n1[3];
  tmc_gradient_f(g, i0, j0, k0, inv, inv2, n0);
  tmc_gradient_f(g, i1, j1, k1, inv, inv2, n1);
  float in[3], scale = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    in[d] = fmaf(l, n1[d] - n0[d], n0[d]);
    scale = fmaxf(scale, fmaxf(fabsf(n0[d]), fabsf(n1[d])));
  }
  const float dot = in[0] * in[0] + in[1] * in[1] + in[2] * in[2];
  // The float32 interpolation errs by a few ulps of `scale`; where the gradients cancel to below
  // 1/16 of it that would exceed ~4e-6 of the unit normal: the reference's float64 normal instead.
  if (scale <= 16.0f * sqrtf(dot)) {
    const float rn = rsqrtf(dot);
#pragma unroll
    for (int d = 0; d < 3; d++) out.n[base + d] = in[d] * rn;
    return;
  }
  double m0[3], m1[3];
  tmc_point_gradient(g, i0, j0, k0, m0);
  tmc_point_gradient(g, i1, j1, k1, m1);
  const double F0d = F0, F1d = F1, ld = (g.iso - F0d) / (F1d - F0d);
  double md[3];
#pragma unroll
  for (int d = 0; d < 3; d++) md[d] = (1 - ld) * m0[d] + ld * m1[d];
  const double nl = sqrt(md[0] * md[0] + md[1] * md[1] + md[2] * md[2]);
#pragma unroll
  for (int d = 0; d < 3; d++) out.n[base + d] = (float)(md[d] / nl);
}

// Vertex index of each crossed edge of a cell, within the cell's volume (vfirst: the volume's first
// vertex in the space-wide numbering; vbase: the cell's first vertex, space-wide).
__device__ __forceinline__ void tmc_vertex_ids(const Grid& g, int i, int j, int k, uint32_t em, uint32_t own,
                                               int32_t vbase, int32_t vfirst, const CellMask* mask,
                                               const uint32_t* rec, const int32_t* voff, int32_t vid[12]) {
#pragma unroll
  for (int e = 0; e < 12; e++) vid[e] = -1;
  // crossed edges as a mask, lowest first: the lanes of a warp resolve their k-th edges together
  for (uint32_t m = em; m; m &= m - 1) {
    const int e = __ffs(m) - 1;
    if (own & (1u << e)) {
      vid[e] = vbase - vfirst + __popc(own & em & ((1u << e) - 1u));
    } else {
      int oi, oj, ok, oe = 0;
      edge_owner(i, j, k, e, oi, oj, ok, oe);
      const uint32_t os = listed_slot(mask, (uint32_t)g.vcell(oi, oj, ok));  // crossed edge: listed owner
      vid[e] = voff[os] - vfirst + __popc(trec_owned(rec[os]) & ((1u << oe) - 1u));
    }
  }
}

// Ambiguous cells, one thread per record of the counting pass: the recorded triangles with the
// cell's vertex indices, and the inner vertices from the recorded parameters (float64 trilinear
// position and normal).  A cell with more triangles than its record holds runs p_slice again.
__global__ void __launch_bounds__(128) tmc_ambiguous_kernel(CellSpace space, const CellMask* mask,
                                                            const uint16_t* cellof, const uint32_t* rec,
                                                            const int32_t* voff, const int32_t* toff,
                                                            const unsigned long long* tile_off, TmcVertexOut out,
                                                            int32_t* tris, const AmbRec* recs, const unsigned* count) {
  const unsigned na = *count;
  for (unsigned a = blockIdx.x * blockDim.x + threadIdx.x; a < na; a += gridDim.x * blockDim.x) {
    const AmbRec& R = recs[a];
    const uint32_t info = R.info;
    if ((info >> 18) & 1) continue;  // singular face: the reference emits nothing for the cell
    const uint32_t slot = R.slot;
    const int64_t vcell = slot_cell(cellof, slot);
    const uint32_t r = rec[slot];
    const Grid g = space.grid_of_tile(vcell / kScanTile);
    const int32_t vfirst = (int32_t)(tile_off[g.vbase / kScanTile] >> 32);
    int i, j, k;
    tcell_ijk(g, vcell - g.vbase, i, j, k);
    const unsigned cs = info & 0xFF;
    const uint32_t em = case_edge_mask(cs);
    const uint32_t own = trec_owned(r);
    int32_t vid[12];
    tmc_vertex_ids(g, i, j, k, em, own, voff[slot], vfirst, mask, rec, voff, vid);
    const int32_t ibase = voff[slot] - vfirst + __popc(own);
    // inner vertices are numbered within the volume: shift the outputs to its first vertex
    InnerOut io{out.v + 3 * (int64_t)vfirst, out.n + 3 * (int64_t)vfirst, out.v64 ? out.v64 + 3 * (int64_t)vfirst : nullptr};
    const int nt = (int)((info >> 8) & 63), ni = (int)((info >> 14) & 7);
    int32_t* t = tris + 3 * (int64_t)toff[slot];
    if ((info >> 17) & 1) {
      float u[8];
      tload_corners(g, i, j, k, u);
      AmbCell amb;
      load_amb_cell(g, i, j, k, u, amb, ni > 0);
      TriSink ts{t, nullptr, 0};
      p_slice_dev(cs, amb.F, g.iso, vid, ibase, ts, amb.P, amb.N, &io, nullptr);
      continue;
    }
    for (int q = 0; q < nt; q++) {
      const unsigned code = R.tri[q];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int x = (int)((code >> (5 * c)) & 31u);
        t[3 * q + c] = x < 12 ? vid[x] : ibase + (x - 12);
      }
    }
    if (ni) {
      // positions in float64 (the output's), normals (float32 outputs only) from float-float
      // gradients; the float64 gradients for float64 outputs and where the gradients cancel
      double P[8][3];
      amb_positions(g, i, j, k, P);
      ffx::ff N[8][3];
      float scale = 0;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        tmc_gradient_ff(g, i + (q & 1), j + ((q >> 1) & 1), k + ((q >> 2) & 1), N[q]);
        scale = fmaxf(scale, fmaxf(fabsf(N[q][0].hi), fmaxf(fabsf(N[q][1].hi), fabsf(N[q][2].hi))));
      }
      double uvw[6][3];
      int nv = 1;
      if (ni == 1) {
        uvw[0][0] = R.prm[0];
        uvw[0][1] = R.prm[1];
        uvw[0][2] = R.prm[2];
      } else {
        const double ui[2] = {R.prm[0], R.prm[1]}, vi[2] = {R.prm[2], R.prm[3]}, wi[2] = {R.prm[4], R.prm[5]};
        hex_corners(ui, vi, wi, uvw);
        nv = 6;
      }
      for (int q = 0; q < nv; q++) {
        // float64 outputs requested for this volume: the reference's float64 normal (and its
        // float32 rounding), as its edge vertices have
        if (!(g.flags & kGridPos64) &&
            inner_vertex_ff(P, N, scale, uvw[q][0], uvw[q][1], uvw[q][2], io, (int64_t)ibase + q))
          continue;
        double Pd[8][3], Nd[8][3];
        amb_geometry(g, i, j, k, Pd, Nd);
        inner_vertex(Pd, Nd, uvw[q][0], uvw[q][1], uvw[q][2], io, (int64_t)ibase + q);
      }
    }
  }
}

// One active cell: its owned edge vertices and (unambiguous case) its table triangles.
template <bool kPos64>
__device__ __forceinline__ void emit_cell(const Grid& g, int32_t vfirst, uint32_t slot, int64_t vcell,
                                          const CellMask* mask, const uint32_t* rec, const int32_t* voff,
                                          const int32_t* toff, const TmcVertexOut& out, int32_t* tris) {
  const int64_t cell = vcell - g.vbase;
  const uint32_t r = rec[slot];
  int i, j, k;
  tcell_ijk(g, cell, i, j, k);
  float u[8];
  tload_corners(g, i, j, k, u);
  unsigned cs = 0;
#pragma unroll
  for (int v = 0; v < 8; v++) cs |= (unsigned)(u[v] >= g.iso_up) << v;
  const uint32_t em = case_edge_mask(cs);
  const uint32_t own = trec_owned(r);
  const int32_t vbase = voff[slot];
  // owned edge vertices, in edge order (the crossed owned edges as a mask, lowest first)
  int rank = 0;
  for (uint32_t mo = em & own; mo; mo &= mo - 1, rank++) {
    const int e = __ffs(mo) - 1;
    if (kPos64 && out.v64 && (g.flags & kGridPos64)) edge_vertex_f64(g, i, j, k, e, u, out, vbase + rank);
    else {
      const float inv2[3] = {g.inv2f[0], g.inv2f[1], g.inv2f[2]};
      const float inv[3] = {2 * inv2[0], 2 * inv2[1], 2 * inv2[2]};  // = fl(1/spacing): doubling is exact
      edge_vertex_f32(g, i, j, k, e, u, out, vbase + rank, inv, inv2);
    }
  }
  // ambiguous: triangles and inner vertices from the cell's ambiguous-cell record (tmc_ambiguous_kernel)
  if ((r >> 21) & 1) return;
  int32_t vid[12];
  tmc_vertex_ids(g, i, j, k, em, own, vbase, vfirst, mask, rec, voff, vid);
  TriSink ts{tris + 3 * (int64_t)toff[slot], 0};
  // unambiguous: table triangles with reversed winding (t_mc, mc/MarchingCubes.cpp:276-294)
  const uint64_t tw = c_tmc_tris[cs];
  const int nt = (int)(tw & 0xF);
  for (int t = 0; t < nt; t++) {
    const int e0 = (int)((tw >> (4 + 12 * t)) & 0xF), e1 = (int)((tw >> (8 + 12 * t)) & 0xF),
              e2 = (int)((tw >> (12 + 12 * t)) & 0xF);
    ts.put(vid[e2], vid[e1], vid[e0]);
  }
}

// Each warp walks chunks of 32 consecutive slots of the listed cells, appends the cells with a
// record to its own queue in shared memory (ballot + popcount), and processes the queue 32 cells at
// a time, one per lane: all lanes busy, and no block barrier (warps never wait for one another).
constexpr int kEmitThreads = 256;
// kPos64: some volume of the launch wants float64 positions (the float64 edge-vertex path is
// compiled only into that instantiation, which keeps the common one's code small)
template <bool kBatch, bool kPos64>
__global__ void __launch_bounds__(kEmitThreads, 4) tmc_emit_kernel(CellSpace space, const CellMask* mask,
                                                                   const uint16_t* cellof, const uint32_t* rec,
                                                                   const int32_t* voff, const int32_t* toff,
                                                                   const unsigned long long* tile_off,
                                                                   TmcVertexOut out, int32_t* tris) {
  constexpr int kWarps = kEmitThreads / 32;
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
      const bool act = r < tile_listed(mask, tile) && rec[slot] != 0;
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (act) Q[qn + __popc(bal & ((1u << lane) - 1u))] = slot;
      qn += __popc(bal);
      __syncwarp();
    }
    while (qn >= 32 || (!more && qn > 0)) {
      const int take = qn < 32 ? qn : 32;
      if (lane < take) {
        const uint32_t slot = Q[lane];
        const uint32_t vcell = slot_cell(cellof, slot);
        // the cell's volume: read in place (a batch's grid table, or the launch parameter)
        const Grid& g = kBatch ? space.grids[__ldg(space.tile_vol + vcell / kScanTile)] : space.one;
        const int32_t vfirst = kBatch ? (int32_t)(tile_off[g.vbase / kScanTile] >> 32) : 0;
        emit_cell<kPos64>(g, vfirst, slot, vcell, mask, rec, voff, toff, out, tris);
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
int64_t tmc_tiles(const CellSpace& space) { return ceil_div(space.n, kScanTile); }

int tmc_classify(const CellSpace& space, TmcScratch& s, cudaStream_t st, Prof* prof, const TileGate* gates,
                 int ngates) {
  const int64_t tiles = tmc_tiles(space);
  // the ambiguous-cell list lives in toff until the offsets kernel overwrites it
  uint32_t* amb_cells = reinterpret_cast<uint32_t*>(s.toff);
  int k = 0;
  {
    Stage t(prof, "tmc_classify", st);
    cudaMemsetAsync(s.amb_n, 0, sizeof(unsigned), st);
    auto classify = [&](int64_t t0, int64_t t1) {
      if (t1 <= t0) return;
      if (space.one.gen)  // fused generation (single volumes)
        tmc_classify_kernel<true><<<(unsigned)(t1 - t0), kScanThreads, 0, st>>>(
            space, t0, s.rec, s.cellof, s.mask, s.tile_sums, s.stats, amb_cells, s.amb_n);
      else
        tmc_classify_kernel<false><<<(unsigned)(t1 - t0), kScanThreads, 0, st>>>(
            space, t0, s.rec, s.cellof, s.mask, s.tile_sums, s.stats, amb_cells, s.amb_n);
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
  }
  return k;
}

int tmc_count(const CellSpace& space, TmcScratch& s, int64_t n_amb, int sms, cudaStream_t st, Prof* prof) {
  const int64_t tiles = tmc_tiles(space);
  const uint32_t* amb_cells = reinterpret_cast<const uint32_t*>(s.toff);
  int k = 0;
  if (n_amb > 0) {
    Stage ta(prof, "tmc_amb_count", st);
    // the list sorted by MC case (the records follow its order, so the emission pass is sorted too)
    const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n_amb, 256), (int64_t)sms * 8));
    cudaMemsetAsync(s.amb_hist, 0, 256 * sizeof(unsigned), st);
    tmc_amb_key_kernel<<<gs, 256, 0, st>>>(space, s.cellof, amb_cells, n_amb, s.amb_key, s.amb_hist);
    tmc_amb_cursor_kernel<<<1, 256, 0, st>>>(s.amb_hist, s.amb_hist + 256);
    tmc_amb_sort_kernel<<<gs, 256, 0, st>>>(amb_cells, s.amb_key, n_amb, s.amb_hist + 256, s.amb_sorted);
    static const int r_amb = resident_blocks(tmc_amb_count_kernel, 128);
    tmc_amb_count_kernel<<<(unsigned)wave_grid(r_amb, sms, 16, n_amb, 128), 128, 0, st>>>(
        space, s.cellof, s.rec, s.tile_sums, s.stats, s.amb_sorted, s.amb_n, reinterpret_cast<AmbRec*>(s.amb_rec));
    k += 4;
  }
  Stage t(prof, "tmc_scan", st);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(s.tile_sums, tiles, s.totals);
  tmc_offsets_kernel<<<(unsigned)ceil_div(tiles, kOffsetWarps), 32 * kOffsetWarps, 0, st>>>(s.mask, s.rec, s.tile_sums,
                                                                                           tiles, s.voff, s.toff);
  return k + 2;
}

int tmc_emit(const CellSpace& space, TmcScratch& s, int64_t n_amb, TmcVertexOut vo, int32_t* tris, const Tuning& tu,
             cudaStream_t st, Prof* prof) {
  const int sms = tu.sms;
  {
    Stage t(prof, "tmc_emit", st);
    const int64_t blocks = std::max<int64_t>(
        1, std::min<int64_t>(ceil_div(space.n, 32 * (kEmitThreads / 32)), (int64_t)sms * tu.emit_blocks_per_sm));
#define TMC_EMIT(B, P)                                                                                       \
  tmc_emit_kernel<B, P><<<(unsigned)blocks, kEmitThreads, 0, st>>>(space, s.mask, s.cellof, s.rec, s.voff, s.toff, \
                                                                  s.tile_sums, vo, tris)
    const bool pos64 = vo.v64 != nullptr;
    if (space.grids) {
      if (pos64) TMC_EMIT(true, true);
      else TMC_EMIT(true, false);
    } else {
      if (pos64) TMC_EMIT(false, true);
      else TMC_EMIT(false, false);
    }
#undef TMC_EMIT
  }
  if (n_amb == 0) return 1;
  Stage t2(prof, "tmc_ambiguous", st);
  static const int r_amb = resident_blocks(tmc_ambiguous_kernel, 128);
  tmc_ambiguous_kernel<<<(unsigned)wave_grid(r_amb, sms, 8, n_amb, 128), 128, 0, st>>>(
      space, s.mask, s.cellof, s.rec, s.voff, s.toff, s.tile_sums, vo, tris, reinterpret_cast<const AmbRec*>(s.amb_rec),
      s.amb_n);
  return 2;
}

}  // namespace tmc
