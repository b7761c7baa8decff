// Halfedge structure of a polygon mesh (quads or triangles), deterministic, as the reference's
// DualMarchingCubes::halfedges builds it (cpp_dmc/DualMarchingCubes.cpp:488-671):
//   halfedge r of face f = index P*f + r (P = 4 or 3): origin = face vertex r, face f,
//   next = P*f + (r+1)%P (all three implicit), twin via the unordered vertex pair of the edge.
// The reference inserts halfedges into a std::map in index order, so within one edge the
// halfedges are ranked by index; an edge with
//   1 halfedge  -> boundary (twin -1)
//   2           -> twins of each other
//   3           -> flag 2 (boundary multiple edge): the pair with different origins are twins,
//                  the third is a boundary halfedge and becomes its origin's handle
//   4           -> flag 1 (non-manifold): paired by origin
// The vertex handle he_v[v] is the last halfedge (in index order) with origin v, overridden by the
// three-halfedge rule in edge-key order (key = min vertex << 32 | max vertex).
//
// GPU scheme: no hash table.  Halfedges are bucketed by origin vertex (counting sort: degree
// count, exclusive scan, scatter of (halfedge, target) pairs), so the halfedges of edge {a, b} are
// the entries of a's list with target b and of b's list with target a.  Vertex lists are short
// (valence ~4) and spatially coherent, so the pairing pass reads mostly from L2.  Sorting the few
// ids of an edge restores the reference's insertion order.  After a simplification pass the
// structure is repaired in place around the vertices the pass touched (repair_halfedges) instead
// of built again.
#include <climits>

#include "halfedges.h"
#include "scan.cuh"

namespace tmc {

namespace {

__global__ void he_vertex_init_kernel(unsigned long long* hv_key, int32_t* deg, int32_t* hv, int64_t nv,
                                      unsigned long long* lone_count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    hv_key[i] = 0;
    deg[i] = 0;
    hv[i] = -1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *lone_count = 0;
}

// out-degrees; the degree counter's old value is the halfedge's slot in its origin's list (one
// atomic per halfedge).  The vertex handle is the highest halfedge with that origin (the
// reference's last insertion): a fire-and-forget atomic maximum.  Twins and flags are written by
// he_twin_kernel, every entry once.
template <bool kHandles>
__global__ void he_build_kernel(const int32_t* faces, int64_t nh, int32_t* deg, int32_t* rank, int32_t* hv) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int v = faces[h];
    rank[h] = atomicAdd(deg + v, 1);
    if (kHandles) atomicMax(hv + v, (int32_t)h);
  }
}

// (at most 32 registers: 8 blocks of 256 threads fit on an SM, the grid's 8 per SM in one wave)
template <int P>  // a compile-time face size: h / P without a run-time 64-bit division
__global__ void __launch_bounds__(256, 8) he_scatter_kernel(const int32_t* faces, int64_t nf, const int32_t* off,
                                                            const int32_t* rank, int2* list) {
  const int64_t nh = nf * P;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int v0 = faces[h], v1 = faces[f * P + (r + 1) % P];
    list[off[v0] + rank[h]] = make_int2((int)h, v1);
  }
}

// The halfedges of the undirected edge {a, b}: returns their number, and the four lowest ids in
// ascending order in id[0..3] (all of them when there are at most four; an edge with more pairs
// none).  Registers only: each id is inserted into the sorted four with fixed compare-swaps.
struct EdgeIds {
  int id[4];
  int c;
};
__device__ __forceinline__ void edge_ids_insert(EdgeIds& e, int x) {
  e.c++;
  if (x >= e.id[3]) return;
  e.id[3] = x;
  if (e.id[3] < e.id[2]) { const int t = e.id[2]; e.id[2] = e.id[3]; e.id[3] = t; }
  if (e.id[2] < e.id[1]) { const int t = e.id[1]; e.id[1] = e.id[2]; e.id[2] = t; }
  if (e.id[1] < e.id[0]) { const int t = e.id[0]; e.id[0] = e.id[1]; e.id[1] = t; }
}
// The list of vertex v is list[off[v] .. off[v + 1]), the last one ends at nh (every halfedge has
// one origin, so the degrees sum to nh): one cache line holds both bounds.
__device__ __forceinline__ int list_end(const int32_t* off, int v, int nv, int nh) {
  return v + 1 < nv ? off[v + 1] : nh;
}

// The twins and flags of a three- or four-halfedge edge {v0, v1} (ids ascending in e), written by
// its lowest halfedge's thread.  kHandles: list the lone halfedge of a three-halfedge edge and its
// key for the vertex handle override.
template <bool kHandles>
__device__ __forceinline__ void resolve_group(const int32_t* faces, const EdgeIds& e, int v0, int v1, int32_t* twin,
                                              uint8_t* flag, unsigned long long* hv_key, int32_t* lone,
                                              unsigned long long* lone_count) {
  if (e.c == 3) {
    const int e0 = e.id[0], e1 = e.id[1], e2 = e.id[2];
    const int a0 = faces[e0], a1 = faces[e1], a2 = faces[e2];
    flag[e0] = 2;
    flag[e1] = 2;
    flag[e2] = 2;
    int lone_v, lone_h;
    if (a0 != a1) {
      twin[e0] = e1; twin[e1] = e0; twin[e2] = -1; lone_v = a2; lone_h = e2;
    } else if (a0 != a2) {
      twin[e0] = e2; twin[e2] = e0; twin[e1] = -1; lone_v = a1; lone_h = e1;
    } else {
      twin[e1] = e2; twin[e2] = e1; twin[e0] = -1; lone_v = a0; lone_h = e0;
    }
    if (kHandles) {
      lone[atomicAdd(lone_count, 1ull)] = lone_h;  // for the handle override
      // the last override in key order wins: remember the largest key (+1 so that 0 = none)
      const unsigned long long key = ((unsigned long long)(unsigned)min(v0, v1) << 32) | (unsigned)max(v0, v1);
      atomicMax(hv_key + lone_v, key + 1ull);
    }
  } else {
    const int e0 = e.id[0], e1 = e.id[1], e2 = e.id[2], e3 = e.id[3];
    if (faces[e0] != faces[e1]) {
      twin[e0] = e1; twin[e1] = e0; twin[e2] = e3; twin[e3] = e2;
    } else {
      twin[e0] = e2; twin[e2] = e0; twin[e1] = e3; twin[e3] = e1;
    }
    flag[e0] = 1; flag[e1] = 1; flag[e2] = 1; flag[e3] = 1;
  }
}

// One thread per face.  The list of corner r's vertex a is read once and serves the face's two
// edges at a: the edge leaving a (halfedges a -> next, forward) and the edge arriving at a (the
// opposite halfedges a -> prev, unless the edge is degenerate, prev == a, whose halfedges are all
// in a's list and counted once as forward).  Per edge the result is the set edge {v_r, v_r+1}
// has, however the face repeats vertices.  Two-halfedge edges pair without coordination; 3 or 4
// are resolved by the edge's lowest halfedge, which writes the twins and flags of all of them;
// every other halfedge is written by its own face (each entry exactly once, as one 16-byte store
// for a quad whose four entries are its own).
template <int P, bool kHandles>
__global__ void he_twin_kernel(const int32_t* faces, int64_t nf, const int2* list, const int32_t* off, int nv,
                               int32_t* twin, uint8_t* flag, unsigned long long* hv_key,
                               unsigned long long* non_manifold, int32_t* lone, unsigned long long* lone_count) {
  const int nh = (int)(nf * P);
  // 16-byte face loads and twin stores only on aligned arrays (a caller's mesh may be a slice)
  const bool vec = P == 4 && ((reinterpret_cast<uintptr_t>(faces) | reinterpret_cast<uintptr_t>(twin)) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(flag) & 3) == 0;
  unsigned long long nm = 0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    int v[P];
    if (vec) {
      const int4 q = reinterpret_cast<const int4*>(faces)[f];
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[P - 1] = q.w;
    } else {
#pragma unroll
      for (int r = 0; r < P; r++) v[r] = faces[P * f + r];
    }
    EdgeIds E[P];
#pragma unroll
    for (int r = 0; r < P; r++) {
      E[r].c = 0;
      E[r].id[0] = E[r].id[1] = E[r].id[2] = E[r].id[3] = INT_MAX;
    }
    // the P corner lists walked in lockstep: P independent loads in flight per step instead of one
    // list after another (the pass is bound by the latency of these gathers)
    int beg[P], len[P], maxlen = 0;
#pragma unroll
    for (int r = 0; r < P; r++) {
      beg[r] = off[v[r]];
      len[r] = list_end(off, v[r], nv, nh) - beg[r];
      maxlen = len[r] > maxlen ? len[r] : maxlen;
    }
    for (int t = 0; t < maxlen; t++) {
      int2 x[P];
#pragma unroll
      for (int r = 0; r < P; r++) x[r] = t < len[r] ? list[beg[r] + t] : make_int2(-1, -1);
#pragma unroll
      for (int r = 0; r < P; r++) {
        if (t >= len[r]) continue;
        const int a = v[r], next = v[(r + 1) % P], prev = v[(r + P - 1) % P];
        if (x[r].y == next) edge_ids_insert(E[r], x[r].x);
        if (x[r].y == prev && prev != a) edge_ids_insert(E[(r + P - 1) % P], x[r].x);
      }
    }
    int tw[P];
    unsigned fl = 0, mine = 0;
#pragma unroll
    for (int r = 0; r < P; r++) {
      const int h = (int)(P * f) + r;
      const EdgeIds& e = E[r];
      tw[r] = -1;
      if (e.c == 2) {
        tw[r] = (e.id[0] == h) ? e.id[1] : e.id[0];
        mine |= 1u << r;
      } else if (e.c < 3 || e.c > 4) {  // boundary, or more halfedges than the rules pair: no twin
        mine |= 1u << r;
      } else if (e.id[0] == h) {
        resolve_group<kHandles>(faces, e, v[r], v[(r + 1) % P], twin, flag, hv_key, lone, lone_count);
        nm++;
      }
    }
    if (vec && mine == 0xfu) {
      reinterpret_cast<int4*>(twin)[f] = make_int4(tw[0], tw[1], tw[2], tw[P - 1]);
      reinterpret_cast<uint32_t*>(flag)[f] = fl;
    } else {
#pragma unroll
      for (int r = 0; r < P; r++)
        if (mine & (1u << r)) {
          twin[P * f + r] = tw[r];
          flag[P * f + r] = 0;
        }
    }
  }
  for (int o = 16; o; o >>= 1) nm += __shfl_down_sync(0xffffffffu, nm, o);
  if ((threadIdx.x & 31) == 0 && nm) atomicAdd(non_manifold, nm);
}

// the lone halfedge of a three-halfedge edge whose key won its origin's override sets the handle
// (the lone halfedges are listed by he_twin_kernel)
__global__ void he_override_kernel(const int32_t* faces, int P, const int32_t* lone, const unsigned long long* lone_count,
                                   int32_t* hv, const unsigned long long* hv_key) {
  const int64_t n = (int64_t)*lone_count;
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
    const int64_t h = lone[a];
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int v0 = faces[h], v1 = faces[f * P + (r + 1) % P];
    const unsigned long long key = ((unsigned long long)(unsigned)min(v0, v1) << 32) | (unsigned)max(v0, v1);
    if (hv_key[v0] == key + 1ull) hv[v0] = (int32_t)h;
  }
}

// ---- repair after a simplification pass (quad meshes, faces and vertices keep their indices) ----
// A pass kills faces and re-targets corners of some live faces.  Call a vertex dirty when a
// re-targeted corner lands on it or it is a corner of a killed face that is still in use: every
// killed face has a dirty or dead end on each of its edges, and every re-targeted corner lands on a
// dirty vertex.  So an edge whose two ends are clean has the same halfedges before and after the
// pass, and keeps its twins and flags as they are.  The live halfedges with a dirty end are bucketed
// by that end (the lower one when both are dirty), so all halfedges of such an edge share one
// bucket, and re-paired there with the build's rules.  Out-degrees of clean vertices are kept (less
// the killed faces' corners, done by the pass); those of dirty vertices are counted here.

// Own twin and flag of halfedge h from its edge's halfedges (ids ascending in e): the rules of
// he_twin_kernel and resolve_group, evaluated by every member for itself.
__device__ __forceinline__ void group_member(const int32_t* faces, const EdgeIds& e, int h, int& tw, int& fl) {
  tw = -1;
  fl = 0;
  if (e.c == 2) {
    tw = (e.id[0] == h) ? e.id[1] : e.id[0];
  } else if (e.c == 3) {
    const int e0 = e.id[0], e1 = e.id[1], e2 = e.id[2];
    const int a0 = faces[e0], a1 = faces[e1], a2 = faces[e2];
    int p = e0, q = e1;  // the twin pair; the third member is the lone boundary halfedge
    if (a0 != a1) {
      p = e0; q = e1;
    } else if (a0 != a2) {
      p = e0; q = e2;
    } else {
      p = e1; q = e2;
    }
    fl = 2;
    tw = (h == p) ? q : (h == q) ? p : -1;
  } else if (e.c == 4) {
    const int e0 = e.id[0], e1 = e.id[1], e2 = e.id[2], e3 = e.id[3];
    // pairs (e0, e1) and (e2, e3), or (e0, e2) and (e1, e3) when e0 and e1 have one origin
    const bool cross = faces[e0] == faces[e1];
    const int a = cross ? e2 : e1, b = cross ? e1 : e2;
    fl = 1;
    tw = (h == e0) ? a : (h == a) ? e0 : (h == b) ? e3 : b;
  }
}

// bucket of a halfedge with a dirty end (origin dirty: dout, target dirty: din)
__device__ __forceinline__ int bucket_of(int o, int t, bool dout, bool din) {
  return (dout && din) ? min(o, t) : (dout ? o : t);
}

// One thread per face: the mask of the live face's halfedges with a dirty end (dmask), their ranks
// in their buckets (drank), and the out-degrees of the dirty vertices (zero on entry).  Quad arrays
// are 16-byte aligned (pool allocations).
__global__ void __launch_bounds__(256) he_repair_mark_kernel(const int4* faces, int64_t nf, const uint8_t* alive,
                                                             const uint8_t* dirty, int32_t* deg, int32_t* bcnt,
                                                             int32_t* drank, uint8_t* dmask) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    unsigned m = 0;
    if (alive[f]) {
      const int4 q = faces[f];
      const int v[4] = {q.x, q.y, q.z, q.w};
      bool d[4];
#pragma unroll
      for (int r = 0; r < 4; r++) d[r] = dirty[v[r]] != 0;
#pragma unroll
      for (int r = 0; r < 4; r++) m |= (unsigned)(d[r] || d[(r + 1) & 3]) << r;
      if (m) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
          if (d[r]) atomicAdd(deg + v[r], 1);
          if (m >> r & 1)
            drank[4 * f + r] = atomicAdd(bcnt + bucket_of(v[r], v[(r + 1) & 3], d[r], d[(r + 1) & 3]), 1);
        }
      }
    }
    dmask[f] = (uint8_t)m;
  }
}

// bucket entries: (halfedge, the edge's other end)
__global__ void he_bucket_scatter_kernel(const int4* faces, int64_t nf, const uint8_t* dirty, const uint8_t* dmask,
                                         const int32_t* drank, const int32_t* boff, int2* blist, int32_t* bkey) {
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    const unsigned m = dmask[f];
    if (!m) continue;
    const int4 q = faces[f];
    const int v[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int r = 0; r < 4; r++) {
      if (!(m >> r & 1)) continue;
      const int o = v[r], t = v[(r + 1) & 3];
      const int key = bucket_of(o, t, dirty[o] != 0, dirty[t] != 0);
      const int at = boff[key] + drank[4 * f + r];
      blist[at] = make_int2((int)(4 * f + r), o == key ? t : o);
      bkey[at] = key;
    }
  }
}

// One thread per bucket entry: its edge is the entries of its bucket with the same other end.  The
// lanes of one bucket load the same entries (one broadcast load per step), all from L1.
__global__ void he_pair_kernel(const int32_t* faces, int nv, const unsigned long long* total, const int32_t* boff,
                               const int2* blist, const int32_t* bkey, int32_t* twin, uint8_t* flag) {
  const int n = (int)*total;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const int2 x = blist[a];
    const int key = bkey[a];
    const int b = boff[key], end = list_end(boff, key, nv, n);
    EdgeIds e;
    e.c = 0;
    e.id[0] = e.id[1] = e.id[2] = e.id[3] = INT_MAX;
    for (int j = b; j < end; j++) {
      const int2 y = blist[j];
      if (y.y == x.y) edge_ids_insert(e, y.x);
    }
    int tw, fl;
    group_member(faces, e, x.x, tw, fl);
    twin[x.x] = tw;
    flag[x.x] = (uint8_t)fl;
  }
}

// Vertex handles and the count of three- and four-halfedge edges from built twins and flags: the
// handle is the highest halfedge with the vertex as origin, overridden by the lone (twinless)
// member of a three-halfedge edge in edge-key order (he_override_kernel).
__global__ void he_handles_init_kernel(int32_t* hv, unsigned long long* hv_key, int64_t nv,
                                       unsigned long long* counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    hv[i] = -1;
    hv_key[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x < 3) counts[threadIdx.x] = 0;
}

template <int P>
__global__ void he_handles_kernel(const int32_t* faces, int64_t nh, const uint8_t* alive, const int32_t* twin,
                                  const uint8_t* flag, int32_t* hv, unsigned long long* hv_key, int32_t* lone,
                                  unsigned long long* counts) {
  unsigned long long n1 = 0, n2 = 0;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    if (alive && !alive[h / P]) continue;
    const int v = faces[h];
    atomicMax(hv + v, (int32_t)h);
    const int fl = flag[h];
    n1 += fl == 1;
    n2 += fl == 2;
    if (fl == 2 && twin[h] == -1) {
      const int64_t f = h / P;
      const int w = faces[f * P + (h - f * P + 1) % P];
      const unsigned long long key = ((unsigned long long)(unsigned)min(v, w) << 32) | (unsigned)max(v, w);
      atomicMax(hv_key + v, key + 1ull);
      lone[atomicAdd(counts + 2, 1ull)] = (int32_t)h;
    }
  }
  for (int o = 16; o; o >>= 1) {
    n1 += __shfl_down_sync(0xffffffffu, n1, o);
    n2 += __shfl_down_sync(0xffffffffu, n2, o);
  }
  if ((threadIdx.x & 31) == 0 && (n1 | n2)) {
    atomicAdd(counts + 0, n1);
    atomicAdd(counts + 1, n2);
  }
}

// The same for quads, one thread per face (16-byte corner and twin loads, the four flags in one word).
__global__ void he_handles4_kernel(const int4* faces, int64_t nf, const uint8_t* alive, const int32_t* twin,
                                   const uint32_t* flag4, int32_t* hv, unsigned long long* hv_key, int32_t* lone,
                                   unsigned long long* counts) {
  unsigned long long n1 = 0, n2 = 0;
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    if (alive && !alive[f]) continue;
    const int4 q = faces[f];
    const uint32_t fw = flag4[f];
    const int v[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int h = (int)(4 * f + r);
      atomicMax(hv + v[r], h);
      const uint32_t fl = (fw >> (8 * r)) & 0xFFu;
      n1 += fl == 1;
      n2 += fl == 2;
      if (fl == 2 && twin[h] == -1) {
        const int w = v[(r + 1) & 3];
        const unsigned long long key = ((unsigned long long)(unsigned)min(v[r], w) << 32) | (unsigned)max(v[r], w);
        atomicMax(hv_key + v[r], key + 1ull);
        lone[atomicAdd(counts + 2, 1ull)] = h;
      }
    }
  }
  for (int o = 16; o; o >>= 1) {
    n1 += __shfl_down_sync(0xffffffffu, n1, o);
    n2 += __shfl_down_sync(0xffffffffu, n2, o);
  }
  if ((threadIdx.x & 31) == 0 && (n1 | n2)) {
    atomicAdd(counts + 0, n1);
    atomicAdd(counts + 1, n2);
  }
}

// edges with four halfedges (flag 1 on each) and with three (flag 2 on each)
__global__ void he_group_count_kernel(const unsigned long long* counts, unsigned long long* non_manifold) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *non_manifold = counts[0] / 4 + counts[1] / 3;
}

// Output records of a compacted quad mesh from halfedges built on its uncompacted form: new face f
// was face src[f], kept face g became fidx[g]; twins move with their faces.
__global__ void he_pack_compacted_kernel(const int32_t* faces, int64_t nh, const int32_t* src, const int32_t* fidx,
                                         const int32_t* twin, int32_t* he4, int32_t* hf) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h >> 2;
    const int r = (int)(h & 3);
    const int T = twin[4 * (int64_t)src[f] + r];
    const int t = T < 0 ? -1 : 4 * fidx[T >> 2] + (T & 3);
    reinterpret_cast<int4*>(he4)[h] = make_int4(faces[h], (int)f, (int)(4 * f + ((r + 1) & 3)), t);
    if (r == 0 && hf) hf[f] = (int32_t)h;
  }
}

// handles of the kept vertices in the compacted numbering (vertex x became vidx[x])
__global__ void he_handles_compacted_kernel(const uint8_t* vkeep, const int32_t* vidx, int64_t nv, const int32_t* hv,
                                            const int32_t* fidx, int32_t* hv_out) {
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < nv; x += (int64_t)gridDim.x * blockDim.x) {
    if (!vkeep[x]) continue;
    const int h = hv[x];
    hv_out[vidx[x]] = h < 0 ? -1 : 4 * fidx[h >> 2] + (h & 3);
  }
}

template <int P>
__global__ void __launch_bounds__(256, 8) he_pack4_kernel(const int32_t* faces, const int32_t* twin, int64_t nh,
                                                          int32_t* he4, int32_t* hf) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    reinterpret_cast<int4*>(he4)[h] = make_int4(faces[h], (int)f, (int)(f * P + (r + 1) % P), twin[h]);
    if (r == 0 && hf) hf[f] = (int32_t)h;
  }
}

}  // namespace

int build_halfedges(const int32_t* faces, int P, int64_t nf, int64_t nv, HeOut& o, HeWork& w, int sms,
                    cudaStream_t st, bool handles) {
  const int64_t nh = nf * P;
  auto grid = [&](int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8));
  };
  int k = 0;
  // the lone-halfedge list reuses the slot array, which is dead once the lists are scattered
  unsigned long long* lone_count = w.total + 1;
  if (handles) {
    he_vertex_init_kernel<<<grid(nv), 256, 0, st>>>(w.hv_key, w.deg, o.hv, nv, lone_count);
    he_build_kernel<true><<<grid(nh), 256, 0, st>>>(faces, nh, w.deg, w.rank, o.hv);
    k += 2;
  } else {
    cudaMemsetAsync(w.deg, 0, (size_t)nv * sizeof(int32_t), st);
    he_build_kernel<false><<<grid(nh), 256, 0, st>>>(faces, nh, w.deg, w.rank, nullptr);
    k += 1;
  }
  k += scan_i32(w.deg, nv, w.off, w.tiles, w.total, st);
  if (P == 4) he_scatter_kernel<4><<<grid(nh), 256, 0, st>>>(faces, nf, w.off, w.rank, w.list);
  else he_scatter_kernel<3><<<grid(nh), 256, 0, st>>>(faces, nf, w.off, w.rank, w.list);
  // one thread per face, whole waves of the kernel's resident blocks
#define HE_TWIN(PP, HH)                                                                                     \
  {                                                                                                         \
    static const int res = resident_blocks(he_twin_kernel<PP, HH>, 256);                                    \
    he_twin_kernel<PP, HH><<<(unsigned)wave_grid(res, sms, 8, nf, 256), 256, 0, st>>>(                       \
        faces, nf, w.list, w.off, (int)nv, o.twin, o.flag, HH ? w.hv_key : nullptr, w.non_manifold,          \
        HH ? w.rank : nullptr, HH ? lone_count : nullptr);                                                  \
  }
  if (P == 4) {
    if (handles) HE_TWIN(4, true) else HE_TWIN(4, false)
  } else {
    if (handles) HE_TWIN(3, true) else HE_TWIN(3, false)
  }
#undef HE_TWIN
  if (handles) {
    he_override_kernel<<<(unsigned)std::max(1, sms), 256, 0, st>>>(faces, P, w.rank, lone_count, o.hv, w.hv_key);
    return k + 3;
  }
  return k + 2;
}

int repair_halfedges(const int32_t* faces, int64_t nf, int64_t nv, const uint8_t* alive, const uint8_t* dirty,
                     HeOut& o, int32_t* deg, HeUpdateWork& w, int sms, cudaStream_t st) {
  if (nf == 0) return 0;
  const int4* q4 = reinterpret_cast<const int4*>(faces);
  cudaMemsetAsync(w.bcnt, 0, (size_t)nv * sizeof(int32_t), st);
  static const int r_mark = resident_blocks(he_repair_mark_kernel, 256);
  he_repair_mark_kernel<<<(unsigned)wave_grid(r_mark, sms, 8, nf, 256), 256, 0, st>>>(q4, nf, alive, dirty, deg, w.bcnt,
                                                                                      w.drank, w.dmask);
  int k = 1 + scan_i32(w.bcnt, nv, w.boff, w.tiles, w.total, st);
  static const int r_sc = resident_blocks(he_bucket_scatter_kernel, 256);
  he_bucket_scatter_kernel<<<(unsigned)wave_grid(r_sc, sms, 8, nf, 256), 256, 0, st>>>(q4, nf, dirty, w.dmask, w.drank,
                                                                                      w.boff, w.blist, w.bkey);
  // the entries are counted on the device: whole waves, as many as the halfedges could need
  static const int r_pair = resident_blocks(he_pair_kernel, 256);
  he_pair_kernel<<<(unsigned)wave_grid(r_pair, sms, 8, 4 * nf, 256), 256, 0, st>>>(faces, (int)nv, w.total, w.boff,
                                                                                  w.blist, w.bkey, o.twin, o.flag);
  return k + 2;
}

int halfedge_handles(const int32_t* faces, int P, int64_t nf, int64_t nv, const uint8_t* alive, const int32_t* twin,
                     const uint8_t* flag, int32_t* hv, HeWork& w, unsigned long long* counts, int sms,
                     cudaStream_t st) {
  const int64_t nh = nf * P;
  auto grid = [&](int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8));
  };
  he_handles_init_kernel<<<grid(nv), 256, 0, st>>>(hv, w.hv_key, nv, counts);
  if (P == 4) {  // quad arrays are 16-byte aligned (pool allocations)
    static const int r4 = resident_blocks(he_handles4_kernel, 256);
    he_handles4_kernel<<<(unsigned)wave_grid(r4, sms, 8, nf, 256), 256, 0, st>>>(
        reinterpret_cast<const int4*>(faces), nf, alive, twin, reinterpret_cast<const uint32_t*>(flag), hv, w.hv_key,
        w.rank, counts);
  } else {
    he_handles_kernel<3><<<grid(nh), 256, 0, st>>>(faces, nh, alive, twin, flag, hv, w.hv_key, w.rank, counts);
  }
  he_override_kernel<<<(unsigned)std::max(1, sms), 256, 0, st>>>(faces, P, w.rank, counts + 2, hv, w.hv_key);
  he_group_count_kernel<<<1, 32, 0, st>>>(counts, w.non_manifold);
  return 4;
}

int pack_compacted_halfedges(const int32_t* faces, int64_t nf, const int32_t* src, const int32_t* fidx,
                             const int32_t* twin, int32_t* he4, int32_t* hf, const uint8_t* vkeep, const int32_t* vidx,
                             int64_t nv, const int32_t* hv, int32_t* hv_out, int sms, cudaStream_t st) {
  auto grid = [&](int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8));
  };
  if (nf > 0) he_pack_compacted_kernel<<<grid(4 * nf), 256, 0, st>>>(faces, 4 * nf, src, fidx, twin, he4, hf);
  he_handles_compacted_kernel<<<grid(nv), 256, 0, st>>>(vkeep, vidx, nv, hv, fidx, hv_out);
  return 2;
}

int pack_halfedges4(const int32_t* faces, int P, const int32_t* twin, int64_t nh, int32_t* he4, int32_t* hf, int sms,
                    cudaStream_t st) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nh, 256), (int64_t)sms * 8));
  if (P == 4) he_pack4_kernel<4><<<g, 256, 0, st>>>(faces, twin, nh, he4, hf);
  else he_pack4_kernel<3><<<g, 256, 0, st>>>(faces, twin, nh, he4, hf);
  return 1;
}

}  // namespace tmc
