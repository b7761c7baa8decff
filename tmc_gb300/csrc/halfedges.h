// Internal interface: deterministic halfedge construction for quad and triangle meshes.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace tmc {

struct HeOut {
  int32_t* he;  // 5 per halfedge: origin, face, next, twin, flag (0 manifold, 1 non-manifold, 2 boundary multiple)
  int32_t* hv;  // per vertex
  int32_t* hf;  // per face
};

// scratch for build_halfedges, sized for nv vertices and nh halfedges
struct HeWork {
  int32_t* deg;                     // nv
  int32_t* off;                     // nv
  int32_t* rank;                    // nh: slot of each halfedge in its origin's list
  int2* list;                       // nh: (halfedge, target vertex) grouped by origin
  unsigned long long* hv_key;       // nv
  unsigned long long* tiles;        // scan_tiles(nv)
  unsigned long long* total;        // 1
  unsigned long long* non_manifold; // 1 (accumulated; zero it before a build)
};

// Returns the number of kernels launched.
int build_halfedges(const int32_t* faces, int P, int64_t nf, int64_t nv, HeOut& o, HeWork& w, int sms,
                    cudaStream_t st);
// {origin, face, next, twin} int4 records for the public output
int pack_halfedges4(const int32_t* he5, int64_t nh, int32_t* he4, int sms, cudaStream_t st);

}  // namespace tmc
