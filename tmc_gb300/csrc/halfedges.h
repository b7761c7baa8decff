// Internal interface: deterministic halfedge construction for quad and triangle meshes.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace tmc {

struct HeTable {
  int64_t size;                // power of two, >= 2 * halfedges
  unsigned long long* keys;    // size
  int32_t* count;              // size
  int32_t* ids;                // 4 * size
};

struct HeOut {
  int32_t* he;  // 5 per halfedge: origin, face, next, twin, flag (0 manifold, 1 non-manifold, 2 boundary multiple)
  int32_t* hv;  // per vertex
  int32_t* hf;  // per face
};

int64_t he_table_size(int64_t nh);
// Returns the number of kernels launched.  hv_key: nv scratch words; slot_of: nf*P scratch ints.
int build_halfedges(const int32_t* faces, int P, int64_t nf, int64_t nv, HeOut& o, HeTable t, int32_t* slot_of,
                    unsigned long long* hv_key, unsigned long long* non_manifold, unsigned* overflow, int sms,
                    cudaStream_t st);
// {origin, face, next, twin} int4 records for the public output
int pack_halfedges4(const int32_t* he5, int64_t nh, int32_t* he4, int sms, cudaStream_t st);

}  // namespace tmc
