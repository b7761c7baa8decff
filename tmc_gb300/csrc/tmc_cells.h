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

constexpr int kTmcAmbRecWords = 32;

struct TmcScratch {
  uint32_t* rec;
  int32_t* voff;
  int32_t* toff;
  unsigned long long* tile_sums;
  unsigned long long* totals;
  unsigned long long* stats;
  unsigned* amb_n;      // ambiguous cells listed by the classification
  uint32_t* amb_rec;    // kTmcAmbRecWords words per ambiguous cell: what the counting pass keeps of
                        // its p_slice for the emission pass (tmc_cells.cu, AmbRec)
  uint32_t* amb_sorted; // the ambiguous cells' slots sorted by MC case (one per ambiguous cell)
  uint8_t* amb_key;     // their cases, in list order (one per ambiguous cell)
  unsigned* amb_hist;   // 512: per-case counts, then scatter cursors
  // listed cells (common.cuh): rec, voff and toff hold one entry per listed cell at its slot, the
  // ambiguous-cell list holds slots
  CellMask* mask;       // per 32 cells of the space
  uint16_t* cellof;     // per slot: in-tile offset of the listed cell
};

// Per-cell scratch is indexed in the cell space; triangles hold vertex indices within their own
// volume, and the volumes' vertices and triangles follow one another in the outputs.
int64_t tmc_tiles(const CellSpace& space);
// Classification: records of the crossed cells and the list of the ambiguous ones, whose number it
// leaves in *s.amb_n.  gates: as dmc_front_count's (classification of a host field arriving in slabs).
int tmc_classify(const CellSpace& space, TmcScratch& s, cudaStream_t st, Prof* prof = nullptr,
                 const TileGate* gates = nullptr, int ngates = 0);
// The ambiguous cells' counts (p_slice, float64) into their records and s.amb_rec (n_amb records,
// n_amb = *s.amb_n), then the vertex and triangle offsets.
int tmc_count(const CellSpace& space, TmcScratch& s, int64_t n_amb, int sms, cudaStream_t st, Prof* prof = nullptr);
int tmc_emit(const CellSpace& space, TmcScratch& s, int64_t n_amb, TmcVertexOut vo, int32_t* tris, const Tuning& tu,
             cudaStream_t st, Prof* prof = nullptr);

}  // namespace tmc
