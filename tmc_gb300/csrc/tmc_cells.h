// Internal interface: topologically correct Marching Cubes kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "profiler.h"

namespace tmc {

struct TmcVertexOut {
  float* v;
  float* n;
  double* v64;  // optional
};

struct TmcScratch {
  uint32_t* rec;
  int32_t* voff;
  int32_t* toff;
  unsigned long long* tile_sums;
  unsigned long long* totals;
  unsigned long long* stats;
  uint32_t* amb_list;   // ambiguous cells with triangles, filled by the emit kernel
  unsigned* amb_count;
  unsigned* amb_n;      // ambiguous cells listed by the classification (count)
  // listed cells (common.cuh): rec, voff and toff hold one entry per listed cell at its slot, the
  // ambiguous lists hold slots
  CellMask* mask;       // per 32 cells of the space
  uint16_t* cellof;     // per slot: in-tile offset of the listed cell
};

// Per-cell scratch is indexed in the cell space; triangles hold vertex indices within their own
// volume, and the volumes' vertices and triangles follow one another in the outputs.
int64_t tmc_tiles(const CellSpace& space);
// gates: as dmc_front_count's (classification of a host field arriving in slabs)
int tmc_count(const CellSpace& space, TmcScratch& s, int sms, cudaStream_t st, Prof* prof = nullptr,
              const TileGate* gates = nullptr, int ngates = 0);
int tmc_emit(const CellSpace& space, TmcScratch& s, TmcVertexOut vo, int32_t* tris, const Tuning& tu, cudaStream_t st,
             Prof* prof = nullptr);

}  // namespace tmc
