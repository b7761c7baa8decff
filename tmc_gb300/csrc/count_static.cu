// tmc_dmc_count_static: the sizes of a Dual Marching Cubes extraction (vertices, quads, active and
// ambiguous cells) computed without allocating any memory.
//
// Who needs it.  Callers that must not allocate device memory at call time: a request server that
// sizes a mesh before admitting the request against a fixed HBM budget (an allocation at that point
// could fail, or grow the memory pool past the budget it is enforcing), or an application that keeps
// its whole device footprint in arenas it sized at start-up.  tmc_dmc_extract cannot serve them: it
// takes its per-cell scratch (records, offsets, tile sums) from the context's memory pool.
//
// How.  A variant of the DMC classification kernel (dmc_front.cu) that keeps no per-cell records:
// each 2048-cell tile writes its packed (vertices << 32 | quads) sum into a file-scope static device
// array, one block adds the tile sums in tile order, and the host reads the totals back.  The
// counts are those of tmc_dmc_extract without simplification (nr_v, nr_q, stats[0], stats[1]).
//
// Limits and sharing.
//  * The static array holds kStaticMaxTiles tile sums: at most 134,217,728 cells (a 513^3-point
//    grid).  Larger grids are rejected with TMC_ERR_CAPACITY before anything is launched.
//  * Every call looks up the array's device address (cudaGetSymbolAddress, with the context's device
//    current); the first call on a device may load this library's device code there, so make that
//    first call before any stream capture on the device.
//  * Every call on a device uses the same array.  Calls that overlap in time on one device (two
//    host threads, or two contexts whose streams are not ordered) race on it and return wrong
//    counts: serialise them.  Each call clears the two cell counters it accumulates atomically;
//    the tile sums and the totals are fully overwritten by every call.
//  * The field must already be in device memory (on_device = 1): copying a host field would need
//    a device buffer.
//  * Nothing is allocated on success; on failure the error message is stored in the context, as
//    for every entry point.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/tmc_gb300.h"
#include "common.cuh"
#include "ctx_access.h"
#include "dmc_cell.cuh"
#include "scan.cuh"

namespace tmc {
namespace {
constexpr int64_t kStaticMaxTiles = 65536;
constexpr int64_t kStaticMaxCells = kStaticMaxTiles * kScanTile;  // 134,217,728
// scratch words: [0, kStaticMaxTiles) tile sums, then the packed total and the two cell counters
constexpr int64_t kTotalWord = kStaticMaxTiles;
constexpr int64_t kActiveWord = kTotalWord + 1;
constexpr int64_t kAmbiguousWord = kTotalWord + 2;
constexpr int64_t kScratchWords = kStaticMaxTiles + 8;  // 512 KiB + 64 B
}  // namespace
}  // namespace tmc

// The scratch of tmc_dmc_count_static (one copy per device, shared by all its calls).
static __device__ __align__(256) unsigned long long tmc_count_scratch[tmc::kScratchWords];

namespace tmc {
namespace {

__constant__ uint64_t c_case_contour_count[256] = TMC_CASE_CONTOUR_INIT;

// Classification without records: one block per tile of kScanTile cells in linear order.
__global__ void __launch_bounds__(kScanThreads) dmc_count_static_kernel(Grid g, unsigned long long* scratch) {
  __shared__ uint64_t cc[256];
  for (int c = threadIdx.x; c < 256; c += blockDim.x) cc[c] = c_case_contour_count[c];
  __syncthreads();
  const int64_t n = g.ncells();
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  unsigned long long local = 0, act = 0, amb = 0;
  for (int s = 0; s < kScanItems; s++) {
    const int64_t c = base + (int64_t)s * kScanThreads + threadIdx.x;
    if (c >= n) break;
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const uint32_t r = classify_cell(g, i, j, k, cc, nullptr);
    local += ((unsigned long long)rec_nv(r) << 32) | (unsigned long long)rec_nq(r);
    act += r != 0;
    amb += (r >> 29) & 1;
  }
  unsigned long long tot;
  block_exclusive_scan<unsigned long long>(local, &tot);
  if (threadIdx.x == 0) scratch[blockIdx.x] = tot;
  for (int o = 16; o; o >>= 1) {
    act += __shfl_down_sync(0xffffffffu, act, o);
    amb += __shfl_down_sync(0xffffffffu, amb, o);
  }
  if ((threadIdx.x & 31) == 0 && (act | amb)) {
    atomicAdd(scratch + kActiveWord, act);
    atomicAdd(scratch + kAmbiguousWord, amb);
  }
}

// Device address of the scratch on the current device.  Looked up on every call: the lookup
// allocates nothing once the module is loaded, and a cudaDeviceReset by the host application (which
// reloads the module, possibly at another address) then cannot leave a stale pointer behind.  The
// mutex serialises the first lookups, which may load this library's device code.
std::mutex g_setup_mutex;

tmc_status scratch_on_device(tmc_ctx* ctx, unsigned long long** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, tmc_count_scratch);
  if (e != cudaSuccess || !p) {
    char msg[256];
    snprintf(msg, sizeof msg, "tmc_dmc_count_static: cudaGetSymbolAddress of the static scratch failed: %s",
             cudaGetErrorString(e));
    return ctx_fail(ctx, TMC_ERR_CUDA, msg);
  }
  *out = static_cast<unsigned long long*>(p);
  return TMC_OK;
}

tmc_status cuda_fail(tmc_ctx* ctx, const char* what, cudaError_t e) {
  char msg[256];
  snprintf(msg, sizeof msg, "tmc_dmc_count_static: %s: %s", what, cudaGetErrorString(e));
  return ctx_fail(ctx, TMC_ERR_CUDA, msg);
}

}  // namespace
}  // namespace tmc

extern "C" tmc_status tmc_dmc_count_static(tmc_ctx* ctx, const tmc_volume* vol, double iso, int64_t counts[4]) {
  using namespace tmc;
  if (!ctx) return TMC_ERR_INVALID_ARG;
  if (!vol || !counts) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "tmc_dmc_count_static: volume or counts is NULL");
  if (!vol->data) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "tmc_dmc_count_static: volume data is NULL");
  if (!vol->on_device)
    return ctx_fail(ctx, TMC_ERR_INVALID_ARG,
                    "tmc_dmc_count_static: the field must be in device memory (on_device = 1); "
                    "copying a host field would allocate");
  if (vol->nx < 2 || vol->ny < 2 || vol->nz < 2 || vol->nx > 65535 || vol->ny > 65535 || vol->nz > 65535)
    return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "tmc_dmc_count_static: every axis needs 2 to 65535 points");
  for (int d = 0; d < 3; d++)
    if (!(vol->spacing[d] > 0) || !std::isfinite(vol->spacing[d]) || !std::isfinite(vol->origin[d]))
      return ctx_fail(ctx, TMC_ERR_INVALID_ARG,
                      "tmc_dmc_count_static: spacing must be positive and finite, the origin finite");
  if (!std::isfinite(iso)) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "tmc_dmc_count_static: iso is not finite");
  const int64_t cells = (int64_t)(vol->nx - 1) * (vol->ny - 1) * (vol->nz - 1);
  if (cells > kStaticMaxCells) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "tmc_dmc_count_static: %lld cells exceed the static scratch limit of %lld cells "
             "(%lld tiles of %d cells); use tmc_dmc_extract for larger grids",
             (long long)cells, (long long)kStaticMaxCells, (long long)kStaticMaxTiles, kScanTile);
    return ctx_fail(ctx, TMC_ERR_CAPACITY, msg);
  }
  const int dev = ctx_device(ctx);
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) return cuda_fail(ctx, "cudaSetDevice", e);
  unsigned long long* scratch = nullptr;
  if (tmc_status s = scratch_on_device(ctx, &scratch)) return s;

  Grid g{};
  g.f = vol->data;
  g.nx = vol->nx;
  g.ny = vol->ny;
  g.nz = vol->nz;
  g.iso = iso;
  float up = (float)iso;
  if ((double)up < iso) up = std::nextafter(up, INFINITY);
  g.iso_up = up;
  g.set_divisors();

  const cudaStream_t st = ctx_stream(ctx);
  const int64_t tiles = ceil_div(cells, kScanTile);
  // the two atomically accumulated cell counters must start at zero
  e = cudaMemsetAsync(scratch + kActiveWord, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return cuda_fail(ctx, "clearing the counters", e);
  dmc_count_static_kernel<<<(unsigned)tiles, kScanThreads, 0, st>>>(g, scratch);
  scan_tile_sums_kernel<<<1, 1024, 0, st>>>(scratch, tiles, scratch + kTotalWord);
  ctx_count_launches(ctx, 2);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, "kernel launch", e);
  unsigned long long h[3] = {0, 0, 0};
  e = cudaMemcpyAsync(h, scratch + kTotalWord, sizeof h, cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(ctx, "reading the totals", e);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(ctx, "cudaStreamSynchronize", e);
  counts[0] = (int64_t)(h[0] >> 32);
  counts[1] = (int64_t)(h[0] & 0xffffffffull);
  counts[2] = (int64_t)h[1];
  counts[3] = (int64_t)h[2];
  return TMC_OK;
}
