// DMC mesh post-processing on the GPU: face colouring, vertex valence, P3X3Y simplification
// (colour pass and isolated pass), P3333 simplification, final halfedges and the quad -> triangle
// split.  Follows cpp_dmc/DualMarchingCubes.cpp:488-1460 step by step; every sequential loop of
// the reference is shown to be order-independent (or made so) where it is parallelised:
//
//  * colorFaces (:714-844): faces are reduced class by class (inherited colours 5..23, then the
//    faces whose inherited colour is 4).  Inherited colour = 3*parity(lower grid point) + axis,
//    and two faces sharing an edge come from two grid edges of one grid face, so they never share
//    an inherited colour: inside one class no face reads another face's new colour.  One launch
//    per class.
//  * mergeVertices3X3Y (:916-1094): a merge reads valence >= 5 vertices and writes valence-3
//    vertices, so reads never see writes.  Several faces writing the same vertex resolve to the
//    highest face index (the reference's last write), via atomicMax claims.
//  * mark3333 (:1189-1322): marked faces cannot be adjacent and their vertices have valence 3, so
//    no vertex is written twice; the neighbour flags are idempotent.
//  * removals (removeVertices3X3Y / removeQuadrilaterals3X3Y, their 3333 pair): the passes run in
//    place, killing faces and re-targeting corners while every index stays; the halfedges are built
//    once and repaired around the touched vertices after each pass (halfedges.cu,
//    repair_halfedges), and one order-preserving compaction after the last pass gives the
//    reference's numbering, since each of its per-pass compactions keeps the order of what remains.
#include <cmath>

#include "../../include/tmc_gb300.h"
#include "dmc_mesh.h"
#include "ffloat.cuh"
#include "halfedges.h"
#include "host_wait.h"
#include "libm_acosf.h"
#include "scan.cuh"

namespace tmc {

namespace {

inline unsigned grid_for(int64_t n, int sms) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8));
}

#define FOR_EACH(i, n) for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// Halfedges of a quad mesh: halfedge r of face f is 4f + r; its origin is quad corner r and its
// next 4f + (r+1)%4 (implicit); twins and flags come from the halfedge build.
struct HeView {
  const int32_t* q;
  const int32_t* twin;
  const uint8_t* flag;
};
__device__ __forceinline__ int he_twin(const HeView& he, int64_t h) { return he.twin[h]; }
__device__ __forceinline__ int he_face(const HeView&, int64_t h) { return (int)(h >> 2); }
__device__ __forceinline__ int he_origin(const HeView& he, int64_t h) { return he.q[h]; }
__device__ __forceinline__ int he_flag(const HeView& he, int64_t h) { return he.flag[h]; }
__device__ __forceinline__ int64_t he_next(int64_t h) { return (h & ~(int64_t)3) | ((h + 1) & 3); }

// collectNeighbors (cpp_dmc/DualMarchingCubes.cpp:673-702); halfedge r of face f is 4f + r
__device__ __forceinline__ void neighbors(const HeView& he, int64_t f, int n[4]) {
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int t = he_twin(he, 4 * f + r);
    n[r] = (t != -1) ? he_face(he, t) : -1;
  }
}

// isNonManifold (:874-885)
__device__ __forceinline__ bool non_manifold(const HeView& he, int64_t f) {
  return he_flag(he, 4 * f) == 1 || he_flag(he, 4 * f + 1) == 1 || he_flag(he, 4 * f + 2) == 1 ||
         he_flag(he, 4 * f + 3) == 1;
}

// ---------------------------------------------------------------------------------------------
// colouring
// ---------------------------------------------------------------------------------------------
// class of an inherited colour: 0..18 for colours 5..23, 19 for colour 4, -1 otherwise
__device__ __forceinline__ int color_class(int c) { return c > 4 ? c - 5 : (c == 4 ? 19 : -1); }

// Class histograms and lists are aggregated per block (shared-memory ranks, one global atomic per
// class and block): 20 global counters hit by every face serialise the whole pass otherwise.  The
// order of faces within a class list does not matter (faces of one class never touch).
constexpr int kColorThreads = 256, kColorItems = 8, kColorTile = kColorThreads * kColorItems;

__global__ void __launch_bounds__(kColorThreads) color_count_kernel(const uint8_t* col, int64_t nq, int32_t* cnt) {
  __shared__ int h[20];
  if (threadIdx.x < 20) h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kColorTile;
#pragma unroll
  for (int s = 0; s < kColorItems; s++) {
    const int64_t f = base + s * kColorThreads + threadIdx.x;
    if (f < nq) {
      const int k = color_class(col[f]);
      if (k >= 0) atomicAdd(&h[k], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x < 20 && h[threadIdx.x]) atomicAdd(cnt + threadIdx.x, h[threadIdx.x]);
}

__global__ void color_offsets_kernel(const int32_t* cnt, int32_t* off, int32_t* cursor) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < 20; k++) {
      off[k] = s;
      cursor[k] = s;
      s += cnt[k];
    }
    off[20] = s;
  }
}

__global__ void __launch_bounds__(kColorThreads) color_scatter_kernel(const uint8_t* col, int64_t nq, int32_t* cursor,
                                                                     int32_t* list) {
  __shared__ int h[20], at[20];
  if (threadIdx.x < 20) h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kColorTile;
  int ks[kColorItems], rs[kColorItems];
#pragma unroll
  for (int s = 0; s < kColorItems; s++) {
    const int64_t f = base + s * kColorThreads + threadIdx.x;
    ks[s] = (f < nq) ? color_class(col[f]) : -1;
    rs[s] = (ks[s] >= 0) ? atomicAdd(&h[ks[s]], 1) : 0;
  }
  __syncthreads();
  if (threadIdx.x < 20 && h[threadIdx.x]) at[threadIdx.x] = atomicAdd(cursor + threadIdx.x, h[threadIdx.x]);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < kColorItems; s++)
    if (ks[s] >= 0) list[at[ks[s]] + rs[s]] = (int32_t)(base + s * kColorThreads + threadIdx.x);
}

__global__ void color_reduce_kernel(HeView he, uint8_t* col, const int32_t* list, const int32_t* off, int k,
                                    int lim) {
  const int64_t b = off[k], e = off[k + 1];
  FOR_EACH(idx, e - b) {
    const int f = list[b + idx];
    int n[4], nc[4];
    neighbors(he, f, n);
#pragma unroll
    for (int r = 0; r < 4; r++) nc[r] = (n[r] != -1) ? (int)col[n[r]] : -1;
    for (int c = 0; c <= lim; c++) {
      if (nc[0] != c && nc[1] != c && nc[2] != c && nc[3] != c) {
        col[f] = (uint8_t)c;
        break;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// valence and patterns
// ---------------------------------------------------------------------------------------------
// vertexValence (:847-871): outgoing halfedges, +1 at the origin of a boundary halfedge's next.
// The outgoing count is the out-degree the halfedge build just counted; only boundary halfedges
// (rare) add with atomics.
// One thread per face (16-byte twin loads; the corners only for a face with a boundary halfedge);
// alive: the live faces (all when NULL).  A caller's quads need not be 16-byte aligned.
__global__ void valence_boundary_kernel(HeView he, int64_t nq, int32_t* val, const uint8_t* alive) {
  const bool vec = ((reinterpret_cast<uintptr_t>(he.q) | reinterpret_cast<uintptr_t>(he.twin)) & 15) == 0;
  FOR_EACH(f, nq) {
    if (alive && !alive[f]) continue;
    const int4 t = vec ? reinterpret_cast<const int4*>(he.twin)[f]
                       : make_int4(he.twin[4 * f], he.twin[4 * f + 1], he.twin[4 * f + 2], he.twin[4 * f + 3]);
    if (t.x != -1 && t.y != -1 && t.z != -1 && t.w != -1) continue;
    const int4 q = vec ? reinterpret_cast<const int4*>(he.q)[f]
                       : make_int4(he.q[4 * f], he.q[4 * f + 1], he.q[4 * f + 2], he.q[4 * f + 3]);
    // a boundary halfedge adds one at the origin of its next, the following corner
    if (t.x == -1) atomicAdd(val + q.y, 1);
    if (t.y == -1) atomicAdd(val + q.z, 1);
    if (t.z == -1) atomicAdd(val + q.w, 1);
    if (t.w == -1) atomicAdd(val + q.x, 1);
  }
}

// mark3X3Y (:889-913)
__global__ void mark3x3y_kernel(const int32_t* q, int64_t nq, const int32_t* val, uint8_t* p, const uint8_t* alive) {
  FOR_EACH(f, nq) {
    if (!alive[f]) {
      p[f] = 0;
      continue;
    }
    const int a = val[q[4 * f]], b = val[q[4 * f + 1]], c = val[q[4 * f + 2]], d = val[q[4 * f + 3]];
    p[f] = (a == 3 && b >= 5 && c == 3 && d >= 5) || (a >= 5 && b == 3 && c >= 5 && d == 3);
  }
}

// mergeVertices3X3Y, both variants (:916-1094): decide removal, claim written vertices
__global__ void merge_claim_kernel(HeView he, int64_t nq, const uint8_t* p, const int32_t* val,
                                   const uint8_t* col, int color_pass, uint8_t* branch, int32_t* own_pos,
                                   int32_t* own_rm) {
  FOR_EACH(f, nq) {
    branch[f] = 0;
    if (!p[f]) continue;
    int n[4];
    neighbors(he, f, n);
    if (color_pass) {
      bool bad = false;
      for (int r = 0; r < 4; r++) {
        if (n[r] >= 0 && non_manifold(he, n[r])) bad = true;
        if (n[r] < 0) bad = true;
      }
      if (bad) continue;
      const int c = col[f];
      bool ok = true;
      for (int r = 0; r < 4; r++)
        if (p[n[r]] && (int)col[n[r]] <= c) ok = false;
      if (!ok) continue;
    } else {
      bool skip = false;
      for (int r = 0; r < 4; r++)
        if (n[r] != -1 && non_manifold(he, n[r])) skip = true;
      for (int r = 0; r < 4; r++)
        if (n[r] != -1 && p[n[r]]) skip = true;
      if (skip) continue;
    }
    const int v0 = he_origin(he, 4 * f), v1 = he_origin(he, 4 * f + 1), v2 = he_origin(he, 4 * f + 2),
              v3 = he_origin(he, 4 * f + 3);
    const int a = val[v0], b = val[v1], c2 = val[v2], d = val[v3];
    if (a == 3 && b >= 5 && c2 == 3 && d >= 5) {
      branch[f] = 1;
      atomicMax(own_pos + v0, (int32_t)f);
      atomicMax(own_rm + v2, (int32_t)f);
    } else if (a >= 5 && b == 3 && c2 >= 5 && d == 3) {
      branch[f] = 2;
      atomicMax(own_pos + v1, (int32_t)f);
      atomicMax(own_rm + v3, (int32_t)f);
    }
  }
}

// The normals kept while simplifying are float pairs (hi, lo) in the 8-byte slots of n64: the front
// end computes them in float-float (within ~2^-40 of the reference's float64 normals), and only their
// float32 roundings leave the library, so they are stored as computed.
__device__ __forceinline__ double pair_to_double(const double* n64, int64_t e) {
  const float2 x = reinterpret_cast<const float2*>(n64)[e];
  return (double)x.x + (double)x.y;
}

// float64 positions and normals: the float32 outputs are their roundings, written once after the
// last pass (float_outputs_kernel)
__device__ __forceinline__ void midpoint(double* v64, double* n64, int dst, int a, int b) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double x = v64[3 * (int64_t)a + d] + 0.5 * (v64[3 * (int64_t)b + d] - v64[3 * (int64_t)a + d]);
    v64[3 * (int64_t)dst + d] = x;
  }
  double m[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double na = pair_to_double(n64, 3 * (int64_t)a + d), nb = pair_to_double(n64, 3 * (int64_t)b + d);
    m[d] = na + 0.5 * (nb - na);
  }
  const double s = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
  float2* n2 = reinterpret_cast<float2*>(n64);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const ffx::ff x = ffx::ff_from_double(m[d] / s);
    n2[3 * (int64_t)dst + d] = make_float2(x.hi, x.lo);
  }
}

// Marks the removed vertices and lists the midpoint merges (destination, two sources); the
// float64 midpoints run densely in midpoint_kernel (a few merging faces per warp would otherwise
// pay the float64 pipe for the whole warp).  Each destination has one owner, and the sources are
// never destinations (valence >= 5 vs valence 3), so the merges are independent.
// dold: the valence-3 corners of the removed faces (merge targets and removed vertices), the
// vertices the halfedge repair re-pairs around; valive: the removed vertices die.
// The jobs of a block's faces are gathered in shared memory and appended with one global atomic
// per block and iteration (per-warp appends to the one counter serialise on it).
constexpr int kMergeThreads = 256;
__global__ void __launch_bounds__(kMergeThreads) merge_apply_kernel(HeView he, int64_t nq, const uint8_t* branch,
                                                                   const int32_t* own_pos, const int32_t* own_rm,
                                                                   uint8_t* vm_first, int32_t* vm_second, uint8_t* em,
                                                                   int4* jobs, unsigned* njobs, uint8_t* dold,
                                                                   uint8_t* valive) {
  __shared__ int4 s_jobs[kMergeThreads];
  __shared__ unsigned s_n, s_base;
  // block-uniform loop: every thread reaches the barriers
  for (int64_t f0 = (int64_t)blockIdx.x * kMergeThreads; f0 < nq; f0 += (int64_t)gridDim.x * kMergeThreads) {
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const int64_t f = f0 + threadIdx.x;
    if (f < nq) {
      const uint8_t br = branch[f];
      em[f] = br != 0;
      if (br) {
        const int v0 = he_origin(he, 4 * f), v1 = he_origin(he, 4 * f + 1), v2 = he_origin(he, 4 * f + 2),
                  v3 = he_origin(he, 4 * f + 3);
        bool job = false;
        int4 jv = make_int4(0, 0, 0, 0);
        if (br == 1) {
          if (own_pos[v0] == f) {
            job = true;
            jv = make_int4(v0, v1, v3, 0);
          }
          dold[v0] = 1;
          dold[v2] = 1;
          vm_first[v2] = 1;
          valive[v2] = 0;
          if (own_rm[v2] == f) vm_second[v2] = v0;
        } else {
          if (own_pos[v1] == f) {
            job = true;
            jv = make_int4(v1, v0, v2, 0);
          }
          dold[v1] = 1;
          dold[v3] = 1;
          vm_first[v3] = 1;
          valive[v3] = 0;
          if (own_rm[v3] == f) vm_second[v3] = v1;
        }
        if (job) s_jobs[atomicAdd(&s_n, 1u)] = jv;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base = s_n ? atomicAdd(njobs, s_n) : 0u;
    __syncthreads();
    if (threadIdx.x < s_n) jobs[s_base + threadIdx.x] = s_jobs[threadIdx.x];
    __syncthreads();  // s_n and s_jobs are read before the next iteration resets them
  }
}

__global__ void midpoint_kernel(const int4* jobs, const unsigned* njobs, double* v64, double* n64) {
  const int64_t nj = *njobs;
  FOR_EACH(a, nj) {
    const int4 j = jobs[a];
    midpoint(v64, n64, j.x, j.y, j.z);
  }
}

// The float32 positions and normals of the simplified mesh: the roundings of its float64 ones (the
// front end writes float32 values that are the same roundings, so that the passes only carry the
// float64 arrays).
__global__ void float_outputs_kernel(const double* v64, const double* n64, int64_t n, float* v, float* nf) {
  const float2* n2 = reinterpret_cast<const float2*>(n64);
  FOR_EACH(e, n) {
    v[e] = (float)v64[e];
    nf[e] = n2[e].x;  // a normalised pair's high part is its float32 rounding
  }
}

// ---------------------------------------------------------------------------------------------
// compaction helpers
// ---------------------------------------------------------------------------------------------

// removeVertices3X3Y / removeVertices3333 (:1096-1112, :1324-1338): kept vertices move to their
// new index, which becomes their map entry.  One thread per vertex component (x, y or z of the
// float64 positions and normals): every load and store is unit-stride across the warp.
// vo, no: the float32 outputs of the kept vertices (the roundings float_outputs_kernel makes), or null
__global__ void gather_vertices_kernel(const uint8_t* keep, const int32_t* idx, int64_t nv, const double* v64,
                                       const double* n64, double* v64o, double* n64o, int32_t* map, int64_t cap,
                                       unsigned* overflow, float* vo, float* no) {
  FOR_EACH(e, 3 * nv) {
    const int64_t i = e / 3;
    if (!keep[i]) continue;
    const int64_t o = idx[i];
    const int d = (int)(e - 3 * i);
    if (o < 0 || o >= cap) {
      if (d == 0) atomicAdd(overflow, 1u);
      continue;
    }
    const double x = v64[e], nn = n64[e];
    v64o[3 * o + d] = x;
    n64o[3 * o + d] = nn;
    if (vo) {
      vo[3 * o + d] = (float)x;
      no[3 * o + d] = reinterpret_cast<const float2*>(n64)[e].x;
    }
    if (d == 0) map[i] = (int32_t)o;
  }
}

// A killed face's corners that stay clean lose one outgoing halfedge each.
__device__ __forceinline__ void killed_face_degrees(const int32_t* q, int64_t f, const uint8_t* dold, int32_t* deg) {
  for (int r = 0; r < 4; r++) {
    const int x = q[4 * f + r];
    if (!dold[x]) atomicSub(deg + x, 1);
  }
}

// Marks a live face's corner x, now y, for the halfedge repair: y is dirty when x was touched by the
// pass (dold), and then its out-degree is recounted from zero.
__device__ __forceinline__ void touch_corner(int x, int y, const uint8_t* dold, uint8_t* dirty, int32_t* deg) {
  if (dold[x] && y >= 0) {
    dirty[y] = 1;
    deg[y] = 0;
  }
}

// removeVertices3X3Y + removeQuadrilaterals3X3Y (:1096-1137) in place: the merged faces die, the
// corners on removed vertices move to their merge target (which a merge always keeps: the faces
// around a valence-3 vertex are pairwise adjacent and no two adjacent faces merge in one pass).
// Faces and vertices keep their indices; the compaction runs once after the last pass.
__global__ void apply_3x3y_kernel(int32_t* q, int64_t nq, uint8_t* alive, const uint8_t* em, const uint8_t* vm_first,
                                  const int32_t* vm_second, const uint8_t* dold, uint8_t* dirty, int32_t* deg) {
  FOR_EACH(f, nq) {
    if (!alive[f]) continue;
    if (em[f]) {
      alive[f] = 0;
      killed_face_degrees(q, f, dold, deg);
      continue;
    }
    for (int r = 0; r < 4; r++) {
      const int x = q[4 * f + r];
      const int y = vm_first[x] ? vm_second[x] : x;
      if (y != x) q[4 * f + r] = y;
      touch_corner(x, y, dold, dirty, deg);
    }
  }
}

// mark3333 (:1189-1322)
__global__ void mark3333_kernel(HeView he, int64_t nq, const int32_t* val, uint8_t* p3, uint8_t* rflag,
                                uint8_t* vm0, int32_t* vm1, uint8_t* dold, const uint8_t* alive, uint8_t* valive) {
  FOR_EACH(f, nq) {
    if (!alive[f] || non_manifold(he, f)) continue;
    int vq[4], fo[4], vo[4];
    for (int r = 0; r < 4; r++) vq[r] = he_origin(he, 4 * f + r);
    if (val[vq[0]] != 3 || val[vq[1]] != 3 || val[vq[2]] != 3 || val[vq[3]] != 3) continue;
    bool boundary = false;
    for (int r = 0; r < 4; r++) {
      const int twin = he_twin(he, 4 * f + r);
      if (twin == -1) {
        boundary = true;
        break;
      }
      fo[r] = he_face(he, twin);
      const int64_t nx = he_next(he_next(twin));
      vo[r] = he_origin(he, nx);
    }
    if (boundary) continue;
    bool nm = false;
    for (int r = 0; r < 4; r++)
      if (non_manifold(he, fo[r])) nm = true;
    if (nm) continue;
    const int a = val[vo[0]], b = val[vo[1]], c = val[vo[2]], d = val[vo[3]];
    if ((a == 3 && b == 3) || (b == 3 && c == 3) || (c == 3 && d == 3) || (d == 3 && a == 3)) continue;
    if (a == 3 || b == 3 || c == 3 || d == 3) continue;
    if (a == 4 && b == 4 && c == 4 && d == 4) continue;
    for (int r = 0; r < 4; r++) {
      vm0[vq[r]] = 1;
      vm1[vq[r]] = vo[r];
      dold[vq[r]] = 1;
      dold[vo[r]] = 1;
      valive[vq[r]] = 0;
    }
    p3[f] = 1;
    for (int r = 0; r < 4; r++) rflag[fo[r]] = 1;
  }
}

// removeVertices3333 + removeQuadrilaterals3333 (:1324-1382) in place: the four neighbours of a
// marked face die and its corners move to the neighbours' far vertices (kept: their valence is not 3).
__global__ void apply_3333_kernel(int32_t* q, int64_t nq, uint8_t* alive, const uint8_t* rflag, const uint8_t* p3,
                                  const int32_t* vm1, const uint8_t* dold, uint8_t* dirty, int32_t* deg) {
  FOR_EACH(f, nq) {
    if (!alive[f]) continue;
    if (rflag[f]) {
      alive[f] = 0;
      killed_face_degrees(q, f, dold, deg);
      continue;
    }
    const bool moved = p3[f] != 0;
    for (int r = 0; r < 4; r++) {
      const int x = q[4 * f + r];
      const int y = moved ? vm1[x] : x;
      if (y != x) q[4 * f + r] = y;
      touch_corner(x, y, dold, dirty, deg);
    }
  }
}

// The live faces at their compacted indices, corners renumbered (vertex x -> vmap[x]); src[o]: the
// face's index before.
__global__ void gather_live_quads_kernel(const uint8_t* alive, const int32_t* idx, int64_t nq, const int32_t* q,
                                         const int32_t* vmap, int32_t* qo, int32_t* src, int64_t cap,
                                         unsigned* overflow) {
  FOR_EACH(f, nq) {
    if (!alive[f]) continue;
    const int64_t o = idx[f];
    if (o < 0 || o >= cap) {
      atomicAdd(overflow, 1u);
      continue;
    }
    src[o] = (int32_t)f;
    for (int r = 0; r < 4; r++) qo[4 * o + r] = vmap[q[4 * f + r]];
  }
}

__global__ void fill_i32_kernel(int32_t* p, int64_t n, int32_t v) {
  FOR_EACH(i, n) p[i] = v;
}

// ---------------------------------------------------------------------------------------------
// quad -> triangles (collectTriangles, :1387-1460; minAngle, DualMarchingCubes.h:746-756)
// ---------------------------------------------------------------------------------------------
// minAngle exactly as the reference: three float arc cosines of the host C library (the restated
// kind of libm_acosf.h that the host's acosf is, bit for bit), float minimum in std::min's order
__device__ __forceinline__ float min_angle_full(float a, float b, float c, int acos_kind) {
  const float A = libm::acosf_kind((b * b + c * c - a * a) / (2 * b * c), acos_kind);
  const float B = libm::acosf_kind((a * a + c * c - b * b) / (2 * a * c), acos_kind);
  const float C = libm::acosf_kind((b * b + a * a - c * c) / (2 * b * a), acos_kind);
  const float mAB = (B < A) ? B : A;
  return (C < mAB) ? C : mAB;
}

__device__ __forceinline__ float side(const double* p, const double* q) {
  const double d = (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]);
  return (float)sqrt(d);
}

__device__ __forceinline__ void write_split(int32_t* t, int64_t i, int v0, int v1, int v2, int v3, bool first) {
  int32_t* o = t + 6 * i;
  if (first) {
    o[0] = v1; o[1] = v3; o[2] = v0; o[3] = v1; o[4] = v2; o[5] = v3;
  } else {
    o[0] = v0; o[1] = v1; o[2] = v2; o[3] = v0; o[4] = v2; o[5] = v3;
  }
}

// Largest cosine of a triangle from float sides with their error bounds, and the bound of the
// result; false when the cosines are not surely inside [-1, 1].
__device__ __forceinline__ bool max_cosine_bounded(float a, float b, float c, float ea, float eb, float ec, float& m,
                                                   float& em) {
  const float cA = (b * b + c * c - a * a) / (2 * b * c);
  const float cB = (a * a + c * c - b * b) / (2 * a * c);
  const float cC = (b * b + a * a - c * c) / (2 * b * a);
  // first-order propagation of the side errors (doubled), plus the rounding of both evaluations
  const float rel = ea / a + eb / b + ec / c;
  const float eA = 2.0f * (2.0f * (a * ea + b * eb + c * ec) / (2 * b * c) + fabsf(cA) * rel) + 0x1p-20f;
  const float eB = 2.0f * (2.0f * (a * ea + b * eb + c * ec) / (2 * a * c) + fabsf(cB) * rel) + 0x1p-20f;
  const float eC = 2.0f * (2.0f * (a * ea + b * eb + c * ec) / (2 * b * a) + fabsf(cC) * rel) + 0x1p-20f;
  if (!(cA - eA >= -1.f && cA + eA <= 1.f && cB - eB >= -1.f && cB + eB <= 1.f && cC - eC >= -1.f &&
        cC + eC <= 1.f))
    return false;
  m = fmaxf(cA, fmaxf(cB, cC));
  em = fmaxf(eA, fmaxf(eB, eC));
  return true;
}

// |p - q| from float positions and a bound of its distance to the reference's float (rounded from
// the float64 length of the float64 difference); each float position is within 2^-24 |x| of its
// float64 value.
__device__ __forceinline__ float side_f(const float* p, const float* q, float& err) {
  const float dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
  const float d = sqrtf(dx * dx + dy * dy + dz * dz);
  const float mag = fabsf(p[0]) + fabsf(q[0]) + fabsf(p[1]) + fabsf(q[1]) + fabsf(p[2]) + fabsf(q[2]);
  err = mag * 0x1p-23f + d * 0x1p-20f;
  return d;
}

// collectTriangles (:1387-1460), first pass: decides the split from the float positions wherever
// the two candidates' smallest angles are apart by more than the error bounds; the other quads are
// listed for the exact pass.
__global__ void triangles_fast_kernel(const int32_t* q, int64_t nq, const float* v, int32_t* t, uint32_t* list,
                                      unsigned* count) {
  const int lane = threadIdx.x & 31;
  FOR_EACH(i, nq) {
    const int v0 = q[4 * i], v1 = q[4 * i + 1], v2 = q[4 * i + 2], v3 = q[4 * i + 3];
    const float *P0 = v + 3 * (int64_t)v0, *P1 = v + 3 * (int64_t)v1, *P2 = v + 3 * (int64_t)v2,
                *P3 = v + 3 * (int64_t)v3;
    float e01, e12, e20, e23, e30, e13;
    const float d01 = side_f(P0, P1, e01), d12 = side_f(P1, P2, e12), d20 = side_f(P2, P0, e20),
                d23 = side_f(P2, P3, e23), d30 = side_f(P3, P0, e30), d13 = side_f(P1, P3, e13);
    float m1, m2, m3, m4, x1, x2, x3, x4;
    bool sure = d01 > 0 && d12 > 0 && d20 > 0 && d23 > 0 && d30 > 0 && d13 > 0 &&
                max_cosine_bounded(d01, d12, d20, e01, e12, e20, m1, x1) &&
                max_cosine_bounded(d20, d23, d30, e20, e23, e30, m2, x2) &&
                max_cosine_bounded(d13, d30, d01, e13, e30, e01, m3, x3) &&
                max_cosine_bounded(d12, d23, d13, e12, e23, e13, m4, x4);
    bool first = false;
    if (sure) {
      // smallest angle of a split = acos of its largest cosine (acos decreasing): the first split
      // (along v1-v3) wins when its largest cosine is smaller
      // The bounds place the reference's largest cosines; a further 2^-20 between them keeps its
      // angles (acos has slope at least 1 in magnitude, and the library's float acos is within one
      // ulp, at most 2^-22 below pi) strictly ordered the same way.
      const float xb = fmaxf(m1, m2), eb = fmaxf(x1, x2), xc = fmaxf(m3, m4), ec = fmaxf(x3, x4);
      if (xb + eb + 0x1p-20f < xc - ec) first = false;       // b1 > c1
      else if (xb - eb > xc + ec + 0x1p-20f) first = true;  // b1 < c1
      else sure = false;
    }
    if (sure) write_split(t, i, v0, v1, v2, v3, first);
    const unsigned am = __activemask();
    const unsigned bal = __ballot_sync(am, !sure);
    if (bal) {
      const int leader = __ffs(bal) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(count, (unsigned)__popc(bal));
      base = __shfl_sync(am, base, leader);
      if (!sure) list[base + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)i;
    }
  }
}

// collectTriangles (:1387-1460), exact pass over the listed quads: the reference's arithmetic
// step by step.  Six side lengths (float of a float64 distance), minAngle of the four triangles with
// the host library's float acos (libm_acosf.h, acos_kind), float64 comparisons of the two splits.
__global__ void triangles_kernel(const int32_t* q, const uint32_t* list, const unsigned* count, const double* v64,
                                 int32_t* t, int acos_kind) {
  const int64_t nl = *count;
  FOR_EACH(a, nl) {
    const int64_t i = list[a];
    const int v0 = q[4 * i], v1 = q[4 * i + 1], v2 = q[4 * i + 2], v3 = q[4 * i + 3];
    const double *P0 = v64 + 3 * (int64_t)v0, *P1 = v64 + 3 * (int64_t)v1, *P2 = v64 + 3 * (int64_t)v2,
                 *P3 = v64 + 3 * (int64_t)v3;
    const float d01 = side(P0, P1), d12 = side(P1, P2), d20 = side(P2, P0), d23 = side(P2, P3), d30 = side(P3, P0),
                d13 = side(P1, P3);
    // triangles (v0,v1,v2), (v0,v2,v3) | (v1,v3,v0), (v1,v2,v3); minAngle(a, b, c) takes the sides
    // |p0p1|, |p1p2|, |p2p0| of its triangle (p0, p1, p2)
    const double a1 = min_angle_full(d01, d12, d20, acos_kind), a2 = min_angle_full(d20, d23, d30, acos_kind);
    const double b1 = a2 < a1 ? a2 : a1, b2 = a1 < a2 ? a2 : a1;
    const double a3 = min_angle_full(d13, d30, d01, acos_kind), a4 = min_angle_full(d12, d23, d13, acos_kind);
    const double c1 = a4 < a3 ? a4 : a3, c2 = a3 < a4 ? a4 : a3;
    write_split(t, i, v0, v1, v2, v3, b1 < c1 || (b1 == c1 && b2 <= c2));
  }
}

// ---------------------------------------------------------------------------------------------
// driver helpers
// ---------------------------------------------------------------------------------------------
struct Pool {
  cudaStream_t st;
  std::vector<void*> temp;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T* get(int64_t n) {
    void* p = nullptr;
    if (err != cudaSuccess) return nullptr;
    err = cudaMallocAsync(&p, (size_t)std::max<int64_t>(n, 4) * sizeof(T), st);
    if (err == cudaSuccess) temp.push_back(p);
    return (T*)p;
  }
  void drop(void* p) {
    for (auto& q : temp)
      if (q == p) q = nullptr;
  }
  ~Pool() {
    for (void* p : temp)
      if (p) cudaFreeAsync(p, st);
  }
};

struct HeBufs {
  int32_t* twin = nullptr;
  uint8_t* flag = nullptr;
  int32_t* hv = nullptr;
  HeWork w{};
  unsigned long long* nm = nullptr;
  unsigned* ovf = nullptr;
  // repairs after the simplification passes: vertices a pass touched (dold) and the dirty ones
  // (dnew); the compacted faces' indices before (src); handle counters
  uint8_t* dold = nullptr;
  uint8_t* dnew = nullptr;
  int32_t* src = nullptr;
  HeUpdateWork u{};
  unsigned long long* hcount = nullptr;
};

// colorFaces (:714-844) on a mesh whose halfedges are built: the inherited colours in `col` become
// the reduced ones, class by class (colours 5..23 to the lowest of 0..4 free among the neighbours,
// then colour 4 to the lowest of 0..3).  Returns the number of kernels launched.
int color_faces(const HeView& he, uint8_t* col, int64_t nq, Pool& pool, int sms, cudaStream_t st) {
  int32_t* cnt = pool.get<int32_t>(24);
  int32_t* off = pool.get<int32_t>(24);
  int32_t* cursor = pool.get<int32_t>(24);
  int32_t* list = pool.get<int32_t>(std::max<int64_t>(nq, 1));
  if (pool.err) return 0;
  cudaMemsetAsync(cnt, 0, 24 * sizeof(int32_t), st);
  const unsigned gc = (unsigned)std::max<int64_t>(1, ceil_div(nq, kColorTile));
  color_count_kernel<<<gc, kColorThreads, 0, st>>>(col, nq, cnt);
  color_offsets_kernel<<<1, 32, 0, st>>>(cnt, off, cursor);
  color_scatter_kernel<<<gc, kColorThreads, 0, st>>>(col, nq, cursor, list);
  const unsigned gq = grid_for(std::max<int64_t>(nq, 1), sms);
  for (int k = 0; k < 19; k++) color_reduce_kernel<<<gq, 256, 0, st>>>(he, col, list, off, k, 4);
  color_reduce_kernel<<<gq, 256, 0, st>>>(he, col, list, off, 19, 3);
  return 23;
}

// vertexValence (:847-871): the out-degrees of the halfedge build plus the boundary corrections
// (alive: the live faces, all when NULL)
int vertex_valence(const HeView& he, const int32_t* deg, int64_t nv, int64_t nq, int32_t* val, int sms,
                   cudaStream_t st, const uint8_t* alive = nullptr) {
  cudaMemcpyAsync(val, deg, nv * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  valence_boundary_kernel<<<grid_for(std::max<int64_t>(nq, 1), sms), 256, 0, st>>>(he, nq, val, alive);
  return 1;
}

HeBufs halfedge_buffers(Pool& pool, int64_t NV, int64_t NQ) {
  HeBufs hw;
  hw.twin = pool.get<int32_t>(4 * NQ);
  hw.flag = pool.get<uint8_t>(4 * NQ);
  hw.hv = pool.get<int32_t>(NV);
  hw.w.deg = pool.get<int32_t>(NV);
  hw.w.off = pool.get<int32_t>(NV);
  hw.w.rank = pool.get<int32_t>(4 * NQ);
  hw.w.list = pool.get<int2>(4 * NQ);
  hw.w.hv_key = pool.get<unsigned long long>(NV);
  hw.w.tiles = pool.get<unsigned long long>(scan_tiles(NV) + 2);
  hw.w.total = pool.get<unsigned long long>(2);
  hw.nm = pool.get<unsigned long long>(2);
  hw.w.non_manifold = hw.nm;
  hw.ovf = pool.get<unsigned>(2);
  hw.hcount = pool.get<unsigned long long>(4);
  return hw;
}

// buffers of the halfedge repairs and of the final compaction
void update_buffers(Pool& pool, HeBufs& hw, int64_t NV, int64_t NQ) {
  hw.dold = pool.get<uint8_t>(NV);
  hw.dnew = pool.get<uint8_t>(NV);
  hw.src = pool.get<int32_t>(NQ);
  hw.u.drank = pool.get<int32_t>(4 * NQ);
  hw.u.dmask = pool.get<uint8_t>(NQ);
  hw.u.bcnt = pool.get<int32_t>(NV);
  hw.u.boff = hw.w.off;    // the build's scratch is idle after the one build
  hw.u.blist = hw.w.list;
  hw.u.bkey = pool.get<int32_t>(4 * NQ);
  hw.u.tiles = hw.w.tiles;
  hw.u.total = hw.w.total;
}

}  // namespace

DmcPostStatus dmc_color_valence(const int32_t* quads, int64_t nq, int64_t nv, uint8_t* colors, int32_t* valence,
                                int sms, cudaStream_t st) {
  DmcPostStatus s;
  if (nq == 0) {
    if (nv > 0) s.err = cudaMemsetAsync(valence, 0, nv * sizeof(int32_t), st);
    return s;
  }
  Pool pool{st};
  HeBufs hw = halfedge_buffers(pool, std::max<int64_t>(nv, 1), nq);
  if ((s.err = pool.err) != cudaSuccess) return s;
  cudaMemsetAsync(hw.nm, 0, 2 * sizeof(unsigned long long), st);
  HeOut ho{hw.twin, hw.flag, hw.hv};
  s.launches += build_halfedges(quads, 4, nq, nv, ho, hw.w, sms, st, false);
  const HeView he{quads, hw.twin, hw.flag};
  s.launches += color_faces(he, colors, nq, pool, sms, st);
  if ((s.err = pool.err) != cudaSuccess) return s;
  s.launches += vertex_valence(he, hw.w.deg, nv, nq, valence, sms, st);
  s.err = cudaGetLastError();
  return s;
}

DmcPostStatus dmc_postprocess(const DmcMesh& in, uint32_t flags, int sms, cudaStream_t st, DmcPostOut* out,
                              unsigned long long* h_cnt, Prof* prof, bool borrowed, const ReadyFn* ready) {
  DmcPostStatus s;
  out->mesh = in;
  const bool c3x3y = flags & TMC_DMC_P3X3Y_COLOR, i3x3y = flags & TMC_DMC_P3X3Y_ISOLATED,
             p3333 = flags & TMC_DMC_P3333, want_t = flags & TMC_OUT_TRIANGLES, want_he = flags & TMC_OUT_HALFEDGES;
  if (!(c3x3y || i3x3y || p3333 || want_t || want_he)) return s;
  // the repairs and handles read quads and flags 4 at a time: front-end meshes are 16-byte aligned
  if (reinterpret_cast<uintptr_t>(in.quads) & 15) {
    s.err = cudaErrorInvalidValue;
    return s;
  }
  Pool pool{st};
  const int64_t NV = std::max<int64_t>(in.nv, 1), NQ = std::max<int64_t>(in.nq, 1);

  DmcMesh cur = in;
  HeBufs hw = halfedge_buffers(pool, NV, NQ);
  unsigned long long* tiles = pool.get<unsigned long long>(scan_tiles(std::max(NV, NQ)) + 2);
  unsigned long long* total = pool.get<unsigned long long>(2);
  if (pool.err) {
    s.err = pool.err;
    return s;
  }
  if (hw.ovf) cudaMemsetAsync(hw.ovf, 0, 2 * sizeof(unsigned), st);
  const unsigned gq = grid_for(NQ, sms), gv = grid_for(NV, sms);
  const bool simplify = (c3x3y || i3x3y || p3333) && in.nq > 0;
  auto build_he = [&](bool handles) {
    Stage tm(prof, "dmc_halfedges", st);
    cudaMemsetAsync(hw.nm, 0, 2 * sizeof(unsigned long long), st);
    HeOut ho{hw.twin, hw.flag, hw.hv};
    s.launches += build_halfedges(cur.quads, 4, cur.nq, cur.nv, ho, hw.w, sms, st, handles);
  };
  auto retire = [&](void* ptr) {
    if (!ptr) return;
    bool mine = false;
    for (auto& q : out->owned)
      if (q == ptr) {
        q = nullptr;
        mine = true;
      }
    if (!mine) out->freed.push_back(ptr);
    if (mine || !borrowed) cudaFreeAsync(ptr, st);
  };
  auto adopt = [&](void* ptr) { out->owned.push_back(ptr); };

  // ---- simplification (simplify3X3Y :1139-1182, simplify3333 :1362-1385) ----
  // In place: faces and vertices keep their indices through the passes (alive / valive flags), the
  // halfedges are built once and repaired after each pass, and one order-preserving compaction after
  // the last pass gives the reference's numbering (each of its per-pass compactions keeps the order
  // of what remains, and every rule that compares indices compares them in the same order).
  bool compacted = false;
  uint8_t *alive = nullptr, *valive = nullptr;
  int32_t *idx = nullptr, *idx_q = nullptr;
  int64_t nv0 = cur.nv, nq0 = cur.nq;  // the uncompacted mesh
  int32_t* q0 = cur.quads;
  if (simplify) {
    update_buffers(pool, hw, NV, NQ);
    int32_t* val = pool.get<int32_t>(NV);
    uint8_t* p = pool.get<uint8_t>(NQ);
    uint8_t* branch = pool.get<uint8_t>(NQ);
    uint8_t* vm_first = pool.get<uint8_t>(NV);
    uint8_t* em = pool.get<uint8_t>(NQ);
    int32_t* own_pos = pool.get<int32_t>(NV);
    int32_t* own_rm = pool.get<int32_t>(NV);
    int32_t* vm_second = pool.get<int32_t>(NV);
    int4* jobs = pool.get<int4>(NQ);
    unsigned* njobs = pool.get<unsigned>(2);
    alive = pool.get<uint8_t>(NQ);
    valive = pool.get<uint8_t>(NV);
    idx = pool.get<int32_t>(NV);
    idx_q = pool.get<int32_t>(NQ);
    if ((s.err = pool.err) != cudaSuccess) return s;
    cudaMemsetAsync(alive, 1, nq0, st);
    cudaMemsetAsync(valive, 1, nv0, st);
    build_he(false);
    const HeView he{q0, hw.twin, hw.flag};
    auto repair = [&]() {
      Stage tm(prof, "dmc_halfedges", st);
      HeOut ho{hw.twin, hw.flag, nullptr};
      s.launches += repair_halfedges(q0, nq0, nv0, alive, hw.dnew, ho, hw.w.deg, hw.u, sms, st);
    };
    // P3X3Y: colour pass, then isolated pass
    for (int pass = 0; pass < 2; pass++) {
      if ((pass == 0 && !c3x3y) || (pass == 1 && !i3x3y)) continue;
      if (pass == 0) {
        Stage tm(prof, "dmc_color", st);
        s.launches += color_faces(he, cur.colors, nq0, pool, sms, st);
        if ((s.err = pool.err) != cudaSuccess) return s;
      }
      {
        Stage tm(prof, "dmc_p3x3y", st);
        s.launches += vertex_valence(he, hw.w.deg, nv0, nq0, val, sms, st, alive);
        mark3x3y_kernel<<<gq, 256, 0, st>>>(q0, nq0, val, p, alive);
        fill_i32_kernel<<<gv, 256, 0, st>>>(own_pos, nv0, -1);
        fill_i32_kernel<<<gv, 256, 0, st>>>(own_rm, nv0, -1);
        fill_i32_kernel<<<gv, 256, 0, st>>>(vm_second, nv0, -1);
        cudaMemsetAsync(vm_first, 0, nv0, st);
        cudaMemsetAsync(hw.dold, 0, nv0, st);
        cudaMemsetAsync(hw.dnew, 0, nv0, st);
        merge_claim_kernel<<<gq, 256, 0, st>>>(he, nq0, p, val, cur.colors, pass == 0, branch, own_pos, own_rm);
        cudaMemsetAsync(njobs, 0, sizeof(unsigned), st);
        merge_apply_kernel<<<gq, kMergeThreads, 0, st>>>(he, nq0, branch, own_pos, own_rm, vm_first, vm_second, em,
                                                         jobs, njobs, hw.dold, valive);
        static const int r_mid = resident_blocks(midpoint_kernel, 256);  // one wave over the merge list
        midpoint_kernel<<<(unsigned)wave_grid(r_mid, sms, 1, nq0, 256), 256, 0, st>>>(jobs, njobs, cur.v64, cur.n64);
        apply_3x3y_kernel<<<gq, 256, 0, st>>>(q0, nq0, alive, em, vm_first, vm_second, hw.dold, hw.dnew, hw.w.deg);
        s.launches += 11;
      }
      repair();
    }
    // P3333
    if (p3333) {
      {
        Stage tm(prof, "dmc_p3333", st);
        uint8_t* p3 = p;
        uint8_t* rflag = em;
        uint8_t* vm0 = vm_first;
        int32_t* vm1 = own_pos;
        s.launches += vertex_valence(he, hw.w.deg, nv0, nq0, val, sms, st, alive);
        cudaMemsetAsync(p3, 0, nq0, st);
        cudaMemsetAsync(rflag, 0, nq0, st);
        cudaMemsetAsync(vm0, 0, nv0, st);
        cudaMemsetAsync(hw.dold, 0, nv0, st);
        cudaMemsetAsync(hw.dnew, 0, nv0, st);
        fill_i32_kernel<<<gv, 256, 0, st>>>(vm1, nv0, -1);
        mark3333_kernel<<<gq, 256, 0, st>>>(he, nq0, val, p3, rflag, vm0, vm1, hw.dold, alive, valive);
        apply_3333_kernel<<<gq, 256, 0, st>>>(q0, nq0, alive, rflag, p3, vm1, hw.dold, hw.dnew, hw.w.deg);
        s.launches += 3;
      }
      repair();
    }
    // the output's vertex handles and edge counts, on the uncompacted mesh (before it is released)
    if (want_he) {
      Stage tm(prof, "dmc_halfedges", st);
      s.launches += halfedge_handles(q0, 4, nq0, nv0, alive, hw.twin, hw.flag, hw.hv, hw.w, hw.hcount, sms, st);
    }
    // ---- the one compaction: live vertices and faces, in order ----
    Stage tm(prof, "dmc_compact", st);
    s.launches += scan_flags(valive, nv0, idx, tiles, total, st);
    s.launches += scan_flags(alive, nq0, idx_q, tiles, total + 1, st);
    cudaMemcpyAsync(h_cnt, total, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    host_wait(st);
    const int64_t nv2 = (int64_t)h_cnt[0], nq2 = (int64_t)h_cnt[1];
    // nothing died: no pass changed the mesh, and it stays as it is (with its halfedges)
    if (nv2 != nv0 || nq2 != nq0) {
      DmcMesh nx = cur;
      void *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr, *qn = nullptr;
      const size_t nvb = (size_t)std::max<int64_t>(nv2, 1) * 3;
      if ((s.err = cudaMallocAsync(&a, nvb * sizeof(double), st)) != cudaSuccess) return s;
      adopt(a);
      if ((s.err = cudaMallocAsync(&b, nvb * sizeof(float), st)) != cudaSuccess) return s;
      adopt(b);
      if ((s.err = cudaMallocAsync(&c, nvb * sizeof(float), st)) != cudaSuccess) return s;
      adopt(c);
      if ((s.err = cudaMallocAsync(&d, nvb * sizeof(double), st)) != cudaSuccess) return s;
      adopt(d);
      if ((s.err = cudaMallocAsync(&qn, (size_t)std::max<int64_t>(nq2, 1) * 4 * sizeof(int32_t), st)) != cudaSuccess)
        return s;
      adopt(qn);
      nx.v64 = (double*)a;
      nx.v = (float*)b;
      nx.n = (float*)c;
      nx.n64 = (double*)d;
      nx.quads = (int32_t*)qn;
      nx.nv = nv2;
      nx.nq = nq2;
      // vertex map into vm_second (free after the passes)
      gather_vertices_kernel<<<grid_for(3 * nv0, sms), 256, 0, st>>>(valive, idx, nv0, cur.v64, cur.n64, nx.v64,
                                                                     nx.n64, vm_second, nv2, hw.ovf, nx.v, nx.n);
      gather_live_quads_kernel<<<gq, 256, 0, st>>>(alive, idx_q, nq0, q0, vm_second, nx.quads, hw.src, nq2, hw.ovf);
      s.launches += 2;
      // the inherited colours are only read by the colour pass; they are not carried along
      retire(cur.v64);
      retire(cur.v);
      retire(cur.n);
      retire(cur.n64);
      retire(cur.quads);
      cur = nx;
      compacted = true;
    }
  }
  // the float32 outputs of the simplified mesh (the compaction's gather writes them when it ran)
  if (s.err == cudaSuccess && simplify && !compacted && cur.nv > 0) {
    float_outputs_kernel<<<grid_for(3 * cur.nv, sms), 256, 0, st>>>(cur.v64, cur.n64, 3 * cur.nv, cur.v, cur.n);
    s.launches += 1;
  }
  // ---- final halfedges and triangles ----
  if (s.err == cudaSuccess && ready) {
    (*ready)(cur.v, (size_t)cur.nv * 3 * sizeof(float));
    (*ready)(cur.n, (size_t)cur.nv * 3 * sizeof(float));
    if (flags & TMC_OUT_POS_F64) (*ready)(cur.v64, (size_t)cur.nv * 3 * sizeof(double));
    (*ready)(cur.quads, (size_t)cur.nq * 4 * sizeof(int32_t));
  }
  if (s.err == cudaSuccess && want_he) {
    if (!simplify) build_he(true);  // the front-end mesh as it is: one build with the handles
    void *he4 = nullptr, *hv = nullptr, *hf = nullptr;
    if ((s.err = cudaMallocAsync(&he4, std::max<int64_t>(4 * cur.nq, 1) * 4 * sizeof(int32_t), st)) == cudaSuccess &&
        (s.err = cudaMallocAsync(&hv, std::max<int64_t>(cur.nv, 1) * sizeof(int32_t), st)) == cudaSuccess &&
        (s.err = cudaMallocAsync(&hf, std::max<int64_t>(cur.nq, 1) * sizeof(int32_t), st)) == cudaSuccess) {
      adopt(he4);
      adopt(hv);
      adopt(hf);
      Stage tm(prof, "dmc_halfedges", st);
      if (compacted) {
        s.launches += pack_compacted_halfedges(cur.quads, cur.nq, hw.src, idx_q, hw.twin, (int32_t*)he4, (int32_t*)hf,
                                               valive, idx, nv0, hw.hv, (int32_t*)hv, sms, st);
      } else {
        s.launches += pack_halfedges4(cur.quads, 4, hw.twin, 4 * cur.nq, (int32_t*)he4, (int32_t*)hf, sms, st);
        cudaMemcpyAsync(hv, hw.hv, cur.nv * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
      }
      if (ready) {
        (*ready)(he4, (size_t)cur.nq * 16 * sizeof(int32_t));
        (*ready)(hv, (size_t)cur.nv * sizeof(int32_t));
        (*ready)(hf, (size_t)cur.nq * sizeof(int32_t));
      }
      cudaMemcpyAsync(h_cnt + 1, hw.nm, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
      host_wait(st);
      out->non_manifold = (int64_t)h_cnt[1];
      out->nhe = 4 * cur.nq;
      out->he = (int32_t*)he4;
      out->he_v = (int32_t*)hv;
      out->he_f = (int32_t*)hf;
    }
  }
  if (s.err == cudaSuccess && want_t) {
    void* tr = nullptr;
    if ((s.err = cudaMallocAsync(&tr, std::max<int64_t>(2 * cur.nq, 1) * 3 * sizeof(int32_t), st)) == cudaSuccess) {
      adopt(tr);
      Stage tm(prof, "dmc_triangles", st);
      uint32_t* tlist = pool.get<uint32_t>(std::max<int64_t>(cur.nq, 1));
      unsigned* tcount = pool.get<unsigned>(2);
      if ((s.err = pool.err) == cudaSuccess) {
        cudaMemsetAsync(tcount, 0, sizeof(unsigned), st);
        triangles_fast_kernel<<<grid_for(cur.nq, sms), 256, 0, st>>>(cur.quads, cur.nq, cur.v, (int32_t*)tr, tlist,
                                                                      tcount);
        triangles_kernel<<<grid_for(cur.nq, sms), 256, 0, st>>>(cur.quads, tlist, tcount, cur.v64, (int32_t*)tr,
                                                                libm::host_acosf_kind());
        s.launches += 2;
        if (ready) (*ready)(tr, (size_t)cur.nq * 6 * sizeof(int32_t));
      }
      out->nt = 2 * cur.nq;
      out->tris = (int32_t*)tr;
    }
  }
  {
    std::vector<void*> keepv;
    for (void* q : out->owned)
      if (q) keepv.push_back(q);
    out->owned.swap(keepv);
  }
  if (s.err == cudaSuccess) s.err = cudaGetLastError();
  out->mesh = cur;
  return s;
}

}  // namespace tmc
