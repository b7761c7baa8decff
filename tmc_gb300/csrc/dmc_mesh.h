// Internal interface: DMC mesh post-processing (halfedges, valence, face colouring, P3X3Y/P3333
// simplification, quad -> triangle split).
#pragma once
#include <cstdint>
#include <functional>
#include <vector>
#include <cuda_runtime.h>

#include "profiler.h"

namespace tmc {

struct DmcMesh {
  int64_t nv = 0, nq = 0;
  float* v = nullptr;
  float* n = nullptr;
  double* v64 = nullptr;
  double* n64 = nullptr;  // normals while simplifying, float pairs (hi, lo) per 8-byte slot (merges average them in float64)
  int32_t* quads = nullptr;
  uint8_t* colors = nullptr;
};

struct DmcPostOut {
  DmcMesh mesh;                 // final vertices and quads
  int64_t nt = 0, nhe = 0;
  int32_t* tris = nullptr;
  int32_t* he = nullptr;        // 4 per halfedge
  int32_t* he_v = nullptr;
  int32_t* he_f = nullptr;
  int64_t non_manifold = 0;
  std::vector<void*> owned;     // new device buffers now owned by the result
  std::vector<void*> freed;     // input buffers released by the post-processing
};

struct DmcPostStatus {
  cudaError_t err = cudaSuccess;
  int launches = 0;
};

// Receives result arrays (device pointer, bytes) as soon as no later kernel of the post-processing
// writes them, in the stream order of `st`: the final vertices (float32 positions and normals, and
// float64 positions with TMC_OUT_POS_F64) and quads before the final halfedges are built, then the
// halfedge arrays, then the triangles.  The caller may start copying them out.
using ReadyFn = std::function<void(const void* dev, size_t bytes)>;

// borrowed: the input arrays belong to the caller (e.g. slices of a batch's shared arrays) and are
// never freed here; they are still listed in out->freed once the result no longer uses them.
// h_staging: pinned host memory for 4 words (counts read back between the passes).
DmcPostStatus dmc_postprocess(const DmcMesh& in, uint32_t flags, int sms, cudaStream_t st, DmcPostOut* out,
                              unsigned long long* h_staging, Prof* prof = nullptr, bool borrowed = false,
                              const ReadyFn* ready = nullptr);

// The face colouring and vertex valence stage alone (colorFaces + vertexValence,
// cpp_dmc/DualMarchingCubes.cpp:714-871): colors holds the inherited colours on entry and the reduced
// ones on return; valence receives one count per vertex.  Device arrays, stream-ordered on `st`.
DmcPostStatus dmc_color_valence(const int32_t* quads, int64_t nq, int64_t nv, uint8_t* colors, int32_t* valence,
                                int sms, cudaStream_t st);

}  // namespace tmc
