// Internal interface between the runtime (C ABI) and the DMC kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "profiler.h"

namespace tmc {

struct DmcVertexOut {
  float* v;        // 3 per vertex
  float* n;        // 3 per vertex
  double* v64;     // optional
  double* n64;     // optional: normals kept while the mesh is simplified, as float pairs (hi, lo) per 8-byte slot
  int64_t* vcell;  // optional (with vuvw)
  float* vuvw;
};

namespace repr {
struct ProjRecord;
}

struct DmcScratch {
  uint32_t* rec;                  // per listed cell (slot)
  int32_t* voff;                  // per listed cell (slot)
  int32_t* qoff;                  // per listed cell (slot)
  uint32_t* vwork;                // per vertex: slot of the generating cell
  unsigned long long* tile_sums;  // per scan tile
  unsigned long long* totals;     // [0] = (vertices << 32) | quads
  unsigned long long* stats;      // 8 counters
  // two-pass vertices (per vertex): projection records, projected points, the one-pass list
  repr::ProjRecord* proj;
  float4* vp;
  uint32_t* fb_list;
  unsigned* fb_count;             // [0] fb_list entries, [1] tail_list entries
  uint32_t* tail_list;            // vertices without a valid 7x7 sample (26x26 retry)
  // listed cells (common.cuh): rec, voff and qoff hold one entry per listed cell at its slot
  CellMask* mask;                 // per 32 cells of the space
  uint16_t* cellof;               // per slot: in-tile offset of the listed cell
  uint8_t* ccase;                 // per slot: the listed cell's MC case
  uint8_t* vrank;                 // per vertex: rank among its cell's vertices (vwork: the cell's slot)
  unsigned* amb_n;                // listed cells with an ambiguous case (their slots wait in qoff)
};
constexpr size_t kProjRecordBytes = 144;  // sizeof(repr::ProjRecord)

// Each launcher returns the number of kernels it launched.
// Per-cell scratch is indexed in the cell space (space.n cells, padding included).
int64_t dmc_tiles(const CellSpace& space);  // scan tiles of the space
// gates: classify the tiles of each gate once its event has completed (a host field arriving in
// slabs); none: the whole field is on the device
int dmc_front_count(const CellSpace& space, DmcScratch& s, cudaStream_t st, Prof* prof = nullptr,
                    const TileGate* gates = nullptr, int ngates = 0);
// Quads hold vertex indices within their own volume; vertices and quads of the volumes follow one
// another in the output arrays.
int dmc_front_emit(const CellSpace& space, DmcScratch& s, DmcVertexOut vo, int64_t nv, int32_t* quads,
                   uint8_t* colors, int flip, const Tuning& tu, cudaStream_t st, Prof* prof = nullptr);

}  // namespace tmc
