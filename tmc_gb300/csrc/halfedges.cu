// Halfedge structure of a polygon mesh (quads or triangles), deterministic, as the reference's
// DualMarchingCubes::halfedges builds it (cpp_dmc/DualMarchingCubes.cpp:488-671):
//   halfedge r of face f = index P*f + r (P = 4 or 3): origin = face vertex r, face f,
//   next = P*f + (r+1)%P, twin via the unordered vertex pair of the edge.
// The reference inserts halfedges into a std::map in index order, so within one edge the
// halfedges are ranked by index; an edge with
//   1 halfedge  -> boundary (twin -1)
//   2           -> twins of each other
//   3           -> flag 2 (boundary multiple edge): the pair with different origins are twins,
//                  the third is a boundary halfedge and becomes its origin's handle
//   4           -> flag 1 (non-manifold): paired by origin
// The vertex handle he_v[v] is the last halfedge (in index order) with origin v, overridden by the
// three-halfedge rule in edge-key order.
//
// GPU scheme: an open-addressing table keyed by the 64-bit unordered vertex pair collects the
// halfedges of every edge (atomic slot append), each bucket then sorts its <= 4 ids, which restores
// the reference's insertion order whatever order the atomics ran in.
#include "halfedges.h"

namespace tmc {

namespace {

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long edge_key(int a, int b) {
  const unsigned lo = (unsigned)min(a, b), hi = (unsigned)max(a, b);
  return ((unsigned long long)lo << 32) | hi;
}

__device__ __forceinline__ uint64_t mix(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

__global__ void he_vertex_init_kernel(int32_t* hv, unsigned long long* hv_key, int64_t nv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    hv[i] = -1;
    if (hv_key) hv_key[i] = 0;
  }
}

// one thread per halfedge: fill the record, vertex handle (max index), insert into the table
__global__ void he_build_kernel(const int32_t* faces, int P, int64_t nf, int32_t* he, int32_t* hv, int32_t* hf,
                                HeTable t, int32_t* slot_of, unsigned* overflow) {
  const int64_t nh = nf * P;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int v0 = faces[h];
    const int v1 = faces[f * P + (r + 1) % P];
    int32_t* e = he + 5 * h;
    e[0] = v0;
    e[1] = (int32_t)f;
    e[2] = (int32_t)(f * P + (r + 1) % P);
    e[3] = -1;
    e[4] = 0;
    if (r == 0) hf[f] = (int32_t)(f * P);
    atomicMax(hv + v0, (int32_t)h);
    const unsigned long long key = edge_key(v0, v1);
    uint64_t b = mix(key) & (uint64_t)(t.size - 1);
    for (int64_t probe = 0; probe < t.size; probe++) {
      const unsigned long long old = atomicCAS(t.keys + b, kEmpty, key);
      if (old == kEmpty || old == key) break;
      b = (b + 1) & (uint64_t)(t.size - 1);
    }
    const int s = atomicAdd(t.count + b, 1);
    if (s < 4) t.ids[4 * b + s] = (int32_t)h;
    else atomicAdd(overflow, 1u);
    slot_of[h] = (int32_t)b;
  }
}

// One thread per halfedge.  Edges with two halfedges (the manifold majority) pair without any
// coordination; an edge with 3 or 4 halfedges is resolved by its lowest halfedge's thread.
__device__ __forceinline__ int sorted_ids(const HeTable& t, int64_t b, int id[4]) {
  const int c = min(t.count[b], 4);
  for (int q = 0; q < 4; q++) id[q] = q < c ? t.ids[4 * b + q] : 0x7fffffff;
  for (int x = 1; x < c; x++)
    for (int y = x; y > 0 && id[y - 1] > id[y]; y--) {
      const int tmp = id[y];
      id[y] = id[y - 1];
      id[y - 1] = tmp;
    }
  return c;
}

__global__ void he_twin_kernel(HeTable t, const int32_t* slot_of, int64_t nh, int32_t* he,
                               unsigned long long* hv_key, unsigned long long* non_manifold) {
  unsigned long long nm = 0;
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = slot_of[h];
    const int cnt = t.count[b];
    if (cnt > 4) continue;  // more than four faces at an edge: left unpaired
#define HE(x) (he + 5 * (int64_t)(x))
    if (cnt == 2) {
      const int a = t.ids[4 * b], c = t.ids[4 * b + 1];
      HE(h)[3] = (a == (int)h) ? c : a;
      continue;
    }
    if (cnt == 1) continue;
    int id[4];
    const int c = sorted_ids(t, b, id);
    if (id[0] != (int)h) continue;  // the lowest halfedge resolves the edge
    if (c == 3) {
      const int e0 = id[0], e1 = id[1], e2 = id[2];
      const int v0 = HE(e0)[0], v1 = HE(e1)[0], v2 = HE(e2)[0];
      HE(e0)[4] = 2;
      HE(e1)[4] = 2;
      HE(e2)[4] = 2;
      int lone_v;
      if (v0 != v1) {
        HE(e0)[3] = e1; HE(e1)[3] = e0; HE(e2)[3] = -1; lone_v = v2;
      } else if (v0 != v2) {
        HE(e0)[3] = e2; HE(e2)[3] = e0; HE(e1)[3] = -1; lone_v = v1;
      } else {
        HE(e1)[3] = e2; HE(e2)[3] = e1; HE(e0)[3] = -1; lone_v = v0;
      }
      // the last override in key order wins: remember the largest key (+1 so that 0 = none)
      atomicMax(hv_key + lone_v, t.keys[b] + 1ull);
      nm++;
    } else if (c == 4) {
      const int e0 = id[0], e1 = id[1], e2 = id[2], e3 = id[3];
      if (HE(e0)[0] != HE(e1)[0]) {
        HE(e0)[3] = e1; HE(e1)[3] = e0; HE(e2)[3] = e3; HE(e3)[3] = e2;
      } else {
        HE(e0)[3] = e2; HE(e2)[3] = e0; HE(e1)[3] = e3; HE(e3)[3] = e1;
      }
      HE(e0)[4] = 1; HE(e1)[4] = 1; HE(e2)[4] = 1; HE(e3)[4] = 1;
      nm++;
    }
#undef HE
  }
  for (int o = 16; o; o >>= 1) nm += __shfl_down_sync(0xffffffffu, nm, o);
  if ((threadIdx.x & 31) == 0 && nm) atomicAdd(non_manifold, nm);
}

// three-halfedge edges whose key won the vertex override write the handle
__global__ void he_override_kernel(HeTable t, const int32_t* slot_of, int64_t nh, const int32_t* he, int32_t* hv,
                                   const unsigned long long* hv_key) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = slot_of[h];
    if (t.count[b] != 3 || he[5 * h + 3] != -1) continue;
    const int v = he[5 * h];
    if (hv_key[v] == t.keys[b] + 1ull) hv[v] = (int32_t)h;
  }
}

__global__ void he_pack4_kernel(const int32_t* he5, int64_t nh, int32_t* he4) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* e = he5 + 5 * h;
    reinterpret_cast<int4*>(he4)[h] = make_int4(e[0], e[1], e[2], e[3]);
  }
}

}  // namespace

// Unique edges are about half the halfedges, so a table of >= nh buckets runs at load ~0.5.
int64_t he_table_size(int64_t nh) {
  int64_t s = 1024;
  while (s < nh) s <<= 1;
  return s;
}

int build_halfedges(const int32_t* faces, int P, int64_t nf, int64_t nv, HeOut& o, HeTable t, int32_t* slot_of,
                    unsigned long long* hv_key, unsigned long long* non_manifold, unsigned* overflow, int sms,
                    cudaStream_t st) {
  const int64_t nh = nf * P;
  auto grid = [&](int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8)); };
  cudaMemsetAsync(t.keys, 0xFF, (size_t)t.size * sizeof(unsigned long long), st);
  cudaMemsetAsync(t.count, 0, (size_t)t.size * sizeof(int32_t), st);
  he_vertex_init_kernel<<<grid(nv), 256, 0, st>>>(o.hv, hv_key, nv);
  he_build_kernel<<<grid(nh), 256, 0, st>>>(faces, P, nf, o.he, o.hv, o.hf, t, slot_of, overflow);
  he_twin_kernel<<<grid(nh), 256, 0, st>>>(t, slot_of, nh, o.he, hv_key, non_manifold);
  he_override_kernel<<<grid(nh), 256, 0, st>>>(t, slot_of, nh, o.he, o.hv, hv_key);
  return 4;
}

int pack_halfedges4(const int32_t* he5, int64_t nh, int32_t* he4, int sms, cudaStream_t st) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nh, 256), (int64_t)sms * 8));
  he_pack4_kernel<<<g, 256, 0, st>>>(he5, nh, he4);
  return 1;
}

}  // namespace tmc
