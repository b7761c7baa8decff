// Internal interface: deterministic halfedge construction for quad and triangle meshes.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace tmc {

// Halfedge h of face f = h / P starts at the face's corner h % P: its origin is faces[h], its next
// is P*f + (h+1)%P.  Only the twin and the flag are stored.
struct HeOut {
  int32_t* twin;  // per halfedge: twin halfedge, -1 on the boundary
  uint8_t* flag;  // per halfedge: 0 manifold, 1 non-manifold (4 halfedges), 2 boundary multiple (3)
  int32_t* hv;    // per vertex: one outgoing halfedge
};

// scratch for build_halfedges, sized for nv vertices and nh halfedges
struct HeWork {
  int32_t* deg;                     // nv
  int32_t* off;                     // nv
  int32_t* rank;                    // nh: slot of each halfedge in its origin's list
  int2* list;                       // nh: (halfedge, target vertex) grouped by origin
  unsigned long long* hv_key;       // nv
  unsigned long long* tiles;        // scan_tiles(nv)
  unsigned long long* total;        // 2: [0] the degree scan total, [1] listed lone halfedges
  unsigned long long* non_manifold; // 1 (accumulated; zero it before a build)
};

// Returns the number of kernels launched.
// handles = false: twins, flags and out-degrees only (o.hv, w.hv_key and the lone list untouched),
// for the simplification passes, which never read the vertex handles.
int build_halfedges(const int32_t* faces, int P, int64_t nf, int64_t nv, HeOut& o, HeWork& w, int sms,
                    cudaStream_t st, bool handles = true);
// scratch for repair_halfedges, sized for nv vertices and nf faces
struct HeUpdateWork {
  int32_t* drank;             // 4 nf: rank of a halfedge with a dirty end in its bucket
  uint8_t* dmask;             // nf: the face's halfedges with a dirty end (bit r: halfedge 4f + r)
  int32_t* bcnt;              // nv: bucket sizes
  int32_t* boff;              // nv: bucket offsets
  int2* blist;                // 4 nf: (halfedge, other end) grouped by bucket
  int32_t* bkey;              // 4 nf: the bucket of each entry
  unsigned long long* tiles;  // scan_tiles(nv)
  unsigned long long* total;  // 2: [0] the halfedges with a dirty end
};

// Twins, flags and out-degrees of a quad mesh after a simplification pass that killed faces
// (alive[f] = 0) and re-targeted corners in place, from those before it (o.twin, o.flag and deg are
// updated in place).  dirty[v]: a re-targeted corner landed on v, or v is a corner of a killed face
// and still in use; deg must hold zero for the dirty vertices and the clean ones' degrees less their
// killed faces.  Twins of live halfedges point to live halfedges.  Quad arrays 16-byte aligned.
// Returns the number of kernels launched.
int repair_halfedges(const int32_t* faces, int64_t nf, int64_t nv, const uint8_t* alive, const uint8_t* dirty,
                     HeOut& o, int32_t* deg, HeUpdateWork& w, int sms, cudaStream_t st);
// Vertex handles (o.hv of build_halfedges) and the count of three- and four-halfedge edges (into
// *w.non_manifold) from built twins and flags, over the faces with alive[f] (all when NULL); counts:
// 3 words of scratch.  Uses w.hv_key and w.rank.
int halfedge_handles(const int32_t* faces, int P, int64_t nf, int64_t nv, const uint8_t* alive, const int32_t* twin,
                     const uint8_t* flag, int32_t* hv, HeWork& w, unsigned long long* counts, int sms,
                     cudaStream_t st);
// Output halfedge records, face handles and vertex handles of a compacted quad mesh (faces: its nf
// quads; new face f was face src[f], kept face g became fidx[g], kept vertex x became vidx[x]) from
// the twins and handles (hv) built on the uncompacted mesh.
int pack_compacted_halfedges(const int32_t* faces, int64_t nf, const int32_t* src, const int32_t* fidx,
                             const int32_t* twin, int32_t* he4, int32_t* hf, const uint8_t* vkeep, const int32_t* vidx,
                             int64_t nv, const int32_t* hv, int32_t* hv_out, int sms, cudaStream_t st);
// {origin, face, next, twin} int4 records and the face handles (first halfedge of each face) of the
// public output
int pack_halfedges4(const int32_t* faces, int P, const int32_t* twin, int64_t nh, int32_t* he4, int32_t* hf, int sms,
                    cudaStream_t st);

}  // namespace tmc
