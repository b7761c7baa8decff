// Host runtime behind the C ABI (include/tmc_gb300.h): contexts, stream-ordered pooled device
// memory, argument checking, and the extraction drivers that sequence the kernels.
#include <atomic>
#include <map>
#include <memory>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tmc_gb300.h"
#include "common.cuh"
#include "ctx_access.h"
#include "dmc.h"
#include "dmc_mesh.h"
#include "ffloat.cuh"
#include "generators.cuh"
#include "halfedges.h"
#include "host_wait.h"
#include "scan.cuh"
#include "profiler.h"
#include "tmc_cells.h"

struct tmc_ctx {
  int device = 0;
  int sms = 0;
  tmc::Tuning tune;                       // launch shapes (defaults from the SM count)
  cudaStream_t stream = nullptr;
  // device-to-host copies of result arrays that are final before the call ends, so that they
  // overlap the call's remaining kernels (created on first use, same priority as `stream`)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_event = nullptr;
  std::vector<cudaEvent_t> slab_events;   // arrival of the slabs of a host field (field_slabs)
  int priority = 0;
  cudaMemPool_t pool = nullptr;
  tmc_ctx_opts opts{};
  std::string err;
  std::atomic<int64_t> launches{0};
  unsigned long long* d_stats = nullptr;  // 8 counters, reused per call
  void* h_pinned = nullptr;               // small pinned staging area (totals, stats)
  tmc::Prof prof;                         // stage timings (off unless enabled)
  // pinned host blocks for TMC_OUT_HOST results, reused across calls; shared by the worker contexts
  // of a request server (tmc::ctx_share_pinned)
  std::shared_ptr<tmc::PinnedPool> pinned = std::make_shared<tmc::PinnedPool>();
  void* pinned_get(size_t bytes) { return pinned->get(bytes); }
  void pinned_put(void* p) { pinned->put(p); }
};

namespace {

// Device arrays shared by the meshes of one batch (each mesh points at its slice); released when
// the last of those meshes is freed.
struct SharedBlock {
  std::vector<void*> dev;
  cudaStream_t stream = nullptr;
  ~SharedBlock() {
    for (void* p : dev) cudaFreeAsync(p, stream);
  }
};

struct MeshPriv {
  std::vector<void*> dev;
  std::vector<void*> host;
  std::shared_ptr<SharedBlock> shared;
};

tmc_status fail(tmc_ctx* ctx, tmc_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return s;
}

#define TMC_CUDA(ctx, call)                                                                     \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? TMC_ERR_OOM : TMC_ERR_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                           \
    }                                                                                           \
  } while (0)

// Stream-ordered allocation from the device's pool; tracked for release.
struct Allocs {
  tmc_ctx* ctx;
  std::vector<void*> ptrs;
  explicit Allocs(tmc_ctx* c) : ctx(c) {}
  ~Allocs() {
    for (void* p : ptrs) cudaFreeAsync(p, ctx->stream);
  }
  template <typename T>
  cudaError_t get(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, count ? count * sizeof(T) : 16, ctx->stream);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = (T*)p;
    return e;
  }
  // hand ownership of p to the caller
  void release(void* p) {
    for (auto& q : ptrs)
      if (q == p) q = nullptr;
    std::vector<void*> keep;
    for (void* q : ptrs)
      if (q) keep.push_back(q);
    ptrs.swap(keep);
  }
};

// The ambiguous cells the TMC classification listed (one host read) and their records for the
// counting pass to fill.
cudaError_t tmc_ambiguous_records(tmc_ctx* ctx, Allocs& al, tmc::TmcScratch& sc, int64_t& n_amb) {
  unsigned* h = (unsigned*)ctx->h_pinned + 320;
  cudaError_t e = cudaMemcpyAsync(h, sc.amb_n, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = tmc::host_wait(ctx->stream);
  if (e != cudaSuccess) return e;
  n_amb = (int64_t)*h;
  const size_t na = (size_t)std::max<int64_t>(n_amb, 1);
  if ((e = al.get(&sc.amb_rec, na * tmc::kTmcAmbRecWords)) != cudaSuccess) return e;
  if ((e = al.get(&sc.amb_sorted, na)) != cudaSuccess) return e;
  if ((e = al.get(&sc.amb_key, na)) != cudaSuccess) return e;
  return al.get(&sc.amb_hist, 512);
}

float iso_up(double iso) {
  float f = (float)iso;
  if ((double)f < iso) f = std::nextafter(f, INFINITY);
  return f;
}

tmc_status check_volume(tmc_ctx* ctx, const tmc_volume* vol) {
  if (!vol) return fail(ctx, TMC_ERR_INVALID_ARG, "volume is NULL");
  if (!vol->data) return fail(ctx, TMC_ERR_INVALID_ARG, "volume data is NULL");
  if (vol->nx < 2 || vol->ny < 2 || vol->nz < 2)
    return fail(ctx, TMC_ERR_INVALID_ARG, "grid %dx%dx%d: every axis needs at least 2 points", vol->nx, vol->ny,
                vol->nz);
  if (vol->nx > 65535 || vol->ny > 65535 || vol->nz > 65535)
    return fail(ctx, TMC_ERR_INVALID_ARG, "grid axis above 65535 points");
  for (int d = 0; d < 3; d++)
    if (!(vol->spacing[d] > 0) || !std::isfinite(vol->spacing[d]) || !std::isfinite(vol->origin[d]))
      return fail(ctx, TMC_ERR_INVALID_ARG, "spacing must be positive and finite");
  const int64_t cells = (int64_t)(vol->nx - 1) * (vol->ny - 1) * (vol->nz - 1);
  if (cells > (int64_t)1 << 32) return fail(ctx, TMC_ERR_INVALID_ARG, "more than 2^32 cells");
  return TMC_OK;
}

// The context's copy stream and its event (created on first use).
cudaError_t ensure_copy_stream(tmc_ctx* ctx) {
  cudaError_t e = cudaSuccess;
  if (!ctx->copy_stream &&
      (e = cudaStreamCreateWithPriority(&ctx->copy_stream, cudaStreamNonBlocking, ctx->priority)) != cudaSuccess)
    return e;
  if (!ctx->copy_event) e = cudaEventCreateWithFlags(&ctx->copy_event, cudaEventDisableTiming);
  return e;
}

// TMC_ERR_NUMERIC: any NaN or Inf in the field sets *flag
__global__ void nonfinite_kernel(const float* f, int64_t n, unsigned* flag) {
  bool bad = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(f[i]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *flag = 1u;
}

// With the context's check_numeric option: fail with TMC_ERR_NUMERIC when the field holds NaN or Inf.
tmc_status check_field_numeric(tmc_ctx* ctx, const float* field, const tmc_volume* vol, Allocs& al) {
  if (!ctx->opts.check_numeric) return TMC_OK;
  const int64_t n = (int64_t)vol->nx * vol->ny * vol->nz;
  unsigned* flag = nullptr;
  TMC_CUDA(ctx, al.get(&flag, 1));
  TMC_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tmc::ceil_div(n, 256), (int64_t)ctx->sms * 8));
  nonfinite_kernel<<<blocks, 256, 0, ctx->stream>>>(field, n, flag);
  ctx->launches += 1;
  unsigned* h = (unsigned*)ctx->h_pinned + 256;
  TMC_CUDA(ctx, cudaMemcpyAsync(h, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  TMC_CUDA(ctx, tmc::host_wait(ctx->stream));
  if (*h) return fail(ctx, TMC_ERR_NUMERIC, "the field holds NaN or Inf");
  return TMC_OK;
}

// Bring the field to the device (copy from host memory when needed).
tmc_status field_on_device(tmc_ctx* ctx, const tmc_volume* vol, Allocs& al, const float** out) {
  const size_t n = (size_t)vol->nx * vol->ny * vol->nz;
  if (vol->on_device) {
    *out = vol->data;
    return check_field_numeric(ctx, *out, vol, al);
  }
  float* d = nullptr;
  TMC_CUDA(ctx, al.get(&d, n));
  TMC_CUDA(ctx, cudaMemcpyAsync(d, vol->data, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  *out = d;
  return check_field_numeric(ctx, *out, vol, al);
}

// A host field for one extraction, copied in z slabs on the copy stream: classification of the
// planes that have arrived runs beside the copy of the rest.  gates[q] holds the scan tiles whose
// cells lie in the planes of slabs 0..q (a cell needs its planes z and z + 1) and the event that
// slab q has arrived.  A device field, a small one, or a context that checks the field for NaN/Inf
// (which needs the whole field first) takes field_on_device and no gates.
// Slab depth and count: the context's tuning (TMC_TUNE_SLAB_MIB, TMC_TUNE_MAX_SLABS).
tmc_status field_slabs(tmc_ctx* ctx, const tmc_volume* vol, Allocs& al, const float** out,
                       std::vector<tmc::TileGate>& gates) {
  gates.clear();
  const size_t plane = (size_t)vol->nx * vol->ny, n = plane * vol->nz;
  const int slabs = (int)std::min<size_t>(
      {(size_t)ctx->tune.max_slabs, n * sizeof(float) / (size_t)ctx->tune.slab_bytes, (size_t)vol->nz / 2});
  if (vol->on_device || ctx->opts.check_numeric || slabs < 2) return field_on_device(ctx, vol, al, out);
  float* d = nullptr;
  TMC_CUDA(ctx, al.get(&d, n));
  TMC_CUDA(ctx, ensure_copy_stream(ctx));
  while ((int)ctx->slab_events.size() < slabs) {
    cudaEvent_t e;
    TMC_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->slab_events.push_back(e);
  }
  // the copies follow the allocation, which is ordered on the context stream
  TMC_CUDA(ctx, cudaEventRecord(ctx->copy_event, ctx->stream));
  TMC_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_event, 0));
  const int64_t cells_per_plane = (int64_t)(vol->nx - 1) * (vol->ny - 1);
  int z0 = 0;
  for (int q = 0; q < slabs; q++) {
    const int z1 = (q == slabs - 1) ? vol->nz : (int)((int64_t)vol->nz * (q + 1) / slabs);
    TMC_CUDA(ctx, cudaMemcpyAsync(d + z0 * plane, vol->data + z0 * plane, (size_t)(z1 - z0) * plane * sizeof(float),
                                  cudaMemcpyHostToDevice, ctx->copy_stream));
    TMC_CUDA(ctx, cudaEventRecord(ctx->slab_events[q], ctx->copy_stream));
    // cells in planes z < z1 - 1 have all eight corners on the device; whole tiles only
    gates.push_back({(int64_t)(z1 - 1) * cells_per_plane / tmc::kScanTile, ctx->slab_events[q]});
    z0 = z1;
  }
  *out = d;
  return TMC_OK;
}

tmc::Grid make_grid(const tmc_volume* vol, const float* dev, double iso) {
  tmc::Grid g{};
  g.f = dev;
  g.nx = vol->nx;
  g.ny = vol->ny;
  g.nz = vol->nz;
  g.ox = vol->origin[0];
  g.oy = vol->origin[1];
  g.oz = vol->origin[2];
  g.dx = vol->spacing[0];
  g.dy = vol->spacing[1];
  g.dz = vol->spacing[2];
  g.iso = iso;
  g.iso_up = iso_up(iso);
  g.inv2[0] = 1.0 / (2 * g.dx);
  g.inv2[1] = 1.0 / (2 * g.dy);
  g.inv2[2] = 1.0 / (2 * g.dz);
  for (int d = 0; d < 3; d++) g.inv2f[d] = (float)g.inv2[d];
  const double org[3] = {g.ox, g.oy, g.oz}, sp[3] = {g.dx, g.dy, g.dz};
  for (int d = 0; d < 3; d++) {
    const tmc::ffx::ff a = tmc::ffx::ff_from_double(org[d]), b = tmc::ffx::ff_from_double(sp[d]);
    g.org_hi[d] = a.hi;
    g.org_lo[d] = a.lo;
    g.sp_hi[d] = b.hi;
    g.sp_lo[d] = b.lo;
    const tmc::ffx::ff c = tmc::ffx::ff_from_double(g.inv2[d]);
    g.inv2_hi[d] = c.hi;
    g.inv2_lo[d] = c.lo;
  }
  g.iso_f = (float)iso;
  g.set_divisors();
  return g;
}

void mesh_reset(tmc_mesh* m) { std::memset(m, 0, sizeof(*m)); }

// per-vertex scratch of the two-pass vertex kernels
cudaError_t dmc_vertex_scratch(Allocs& al, tmc::DmcScratch& sc, int64_t nv) {
  uint8_t* rec = nullptr;
  cudaError_t e = al.get(&rec, nv * (int64_t)tmc::kProjRecordBytes);
  sc.proj = reinterpret_cast<tmc::repr::ProjRecord*>(rec);
  if (e == cudaSuccess) e = al.get(&sc.vp, nv);
  if (e == cudaSuccess) e = al.get(&sc.fb_list, nv);
  if (e == cudaSuccess) e = al.get(&sc.fb_count, 2);
  if (e == cudaSuccess) e = al.get(&sc.tail_list, nv);
  return e;
}

// Early device-to-host copies for TMC_OUT_HOST: an array handed to issue() is final (no later
// kernel of the call writes it), so its copy starts on the context's copy stream, after the work
// queued so far on the context stream, and runs beside the call's remaining kernels.
// finish_mesh then takes the host block from here instead of copying the array again.
struct EarlyCopies {
  tmc_ctx* ctx = nullptr;
  MeshPriv* mp = nullptr;
  std::vector<std::pair<const void*, void*>> done;  // device array -> pinned host block
  cudaError_t err = cudaSuccess;

  void issue(const void* dev, size_t bytes) {
    if (!dev || !bytes || err != cudaSuccess || host_of(dev)) return;
    if ((err = ensure_copy_stream(ctx)) != cudaSuccess) return;
    void* h = ctx->pinned_get(bytes);
    if (!h) {
      err = cudaErrorMemoryAllocation;
      return;
    }
    mp->host.push_back(h);
    if ((err = cudaEventRecord(ctx->copy_event, ctx->stream)) != cudaSuccess ||
        (err = cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_event, 0)) != cudaSuccess ||
        (err = cudaMemcpyAsync(h, dev, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream)) != cudaSuccess)
      return;
    done.emplace_back(dev, h);
  }
  void* host_of(const void* dev) const {
    for (const auto& d : done)
      if (d.first == dev) return d.second;
    return nullptr;
  }
  // the context stream waits for the copies issued so far
  cudaError_t join() {
    if (done.empty()) return err;
    if (err == cudaSuccess) err = cudaEventRecord(ctx->copy_event, ctx->copy_stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(ctx->stream, ctx->copy_event, 0);
    return err;
  }
};

// Move device arrays of a finished mesh to host memory when TMC_OUT_HOST is set.
template <typename T>
tmc_status to_host(tmc_ctx* ctx, T** p, size_t count, MeshPriv* mp, const EarlyCopies* early) {
  if (!*p) return TMC_OK;
  if (early) {
    if (void* e = early->host_of(*p)) {
      *p = (T*)e;
      return TMC_OK;
    }
  }
  T* h = (T*)ctx->pinned_get(count ? count * sizeof(T) : 16);
  if (!h) return fail(ctx, TMC_ERR_OOM, "host allocation of %zu bytes failed", count * sizeof(T));
  if (count) TMC_CUDA(ctx, cudaMemcpyAsync(h, *p, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  mp->host.push_back(h);
  *p = h;
  return TMC_OK;
}

tmc_status finish_mesh(tmc_ctx* ctx, uint32_t flags, tmc_mesh* out, MeshPriv* mp, EarlyCopies* early = nullptr) {
  tmc_status s = TMC_OK;
  if (flags & TMC_OUT_HOST) {
    const size_t nv = (size_t)out->nr_v, nq = (size_t)out->nr_q, nt = (size_t)out->nr_t, nh = (size_t)out->nr_he;
    if ((s = to_host(ctx, &out->v, 3 * nv, mp, early))) return s;
    if ((s = to_host(ctx, &out->n, 3 * nv, mp, early))) return s;
    if ((s = to_host(ctx, &out->v64, 3 * nv, mp, early))) return s;
    if ((s = to_host(ctx, &out->quads, 4 * nq, mp, early))) return s;
    if ((s = to_host(ctx, &out->tris, 3 * nt, mp, early))) return s;
    if ((s = to_host(ctx, &out->he, 4 * nh, mp, early))) return s;
    if ((s = to_host(ctx, &out->he_v, nv, mp, early))) return s;
    if ((s = to_host(ctx, &out->he_f, out->nr_q ? nq : nt, mp, early))) return s;
    if ((s = to_host(ctx, &out->vcell, nv, mp, early))) return s;
    if ((s = to_host(ctx, &out->vuvw, 3 * nv, mp, early))) return s;
    if (early) TMC_CUDA(ctx, early->join());
    TMC_CUDA(ctx, tmc::host_wait(ctx->stream));
    for (void* p : mp->dev) cudaFreeAsync(p, ctx->stream);
    mp->dev.clear();
    mp->shared.reset();
    out->on_device = 0;
  } else {
    out->on_device = 1;
  }
  out->priv = mp;
  return TMC_OK;
}

// Fused generation: the field buffer comes from the call's pool and the classification writes it
// (Grid::gen_out) while it evaluates the generator; vol describes the generated grid (no data).
struct FusedGen {
  tmc::GenParams params;
  float d[3];
};

// The volume of a generator's grid (origin -1, the float32 spacing), checked
tmc_status gen_volume(tmc_ctx* ctx, const tmc_generator* gen, FusedGen& fg, tmc_volume& vol) {
  if (!gen || !tmc::gen_params(*gen, fg.params, fg.d))
    return fail(ctx, TMC_ERR_INVALID_ARG, "invalid generator (surface, grid or parameters)");
  vol = tmc_volume{};
  vol.nx = gen->nx;
  vol.ny = gen->ny;
  vol.nz = gen->nz;
  for (int a = 0; a < 3; a++) {
    vol.origin[a] = -1.0;
    vol.spacing[a] = (double)fg.d[a];
  }
  vol.on_device = 1;
  const int64_t cells = (int64_t)(vol.nx - 1) * (vol.ny - 1) * (vol.nz - 1);
  if (cells > (int64_t)1 << 32) return fail(ctx, TMC_ERR_INVALID_ARG, "more than 2^32 cells");
  return TMC_OK;
}

// The generated field's buffer (written by the classification) and the grid's generator fields.
tmc_status fused_field(tmc_ctx* ctx, const tmc_volume* vol, const FusedGen& fg, Allocs& al, const float** field,
                       tmc::GenParams** dev_params) {
  float* buf = nullptr;
  TMC_CUDA(ctx, al.get(&buf, (int64_t)vol->nx * vol->ny * vol->nz));
  tmc::GenParams P = fg.params;
  if (tmc::axis_separable(P.surface)) {
    float2* tab = nullptr;
    const int total = vol->nx + vol->ny + vol->nz;
    TMC_CUDA(ctx, al.get(&tab, total));
    tmc::axis_terms_kernel<<<(unsigned)tmc::ceil_div(total, 256), 256, 0, ctx->stream>>>(P, vol->nx, vol->ny, vol->nz,
                                                                                   fg.d[0], fg.d[1], fg.d[2], tab);
    ctx->launches += 1;
    TMC_CUDA(ctx, cudaGetLastError());
    P.tab[0] = tab;
    P.tab[1] = tab + vol->nx;
    P.tab[2] = tab + vol->nx + vol->ny;
  }
  TMC_CUDA(ctx, al.get(dev_params, 1));
  // pageable source: the copy is staged before the call returns, so P may go out of scope
  TMC_CUDA(ctx, cudaMemcpyAsync(*dev_params, &P, sizeof(tmc::GenParams), cudaMemcpyHostToDevice, ctx->stream));
  *field = buf;
  return TMC_OK;
}
void set_fused(tmc::Grid& g, const FusedGen& fg, tmc::GenParams* dev_params) {
  g.gen = dev_params;
  g.gen_out = const_cast<float*>(g.f);
  for (int a = 0; a < 3; a++) g.gd[a] = fg.d[a];
}

tmc_status dmc_extract(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out,
                       const FusedGen* fg);

}  // namespace

// ============================================================================================
// C ABI
// ============================================================================================
extern "C" {

tmc_status tmc_ctx_create(int device, const tmc_ctx_opts* opts, tmc_ctx** out) {
  if (!out) return TMC_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return TMC_ERR_CUDA;
  if (device < 0 || device >= ndev) return TMC_ERR_INVALID_ARG;
  tmc_ctx* ctx = new (std::nothrow) tmc_ctx();
  if (!ctx) return TMC_ERR_OOM;
  ctx->device = device;
  if (opts) ctx->opts = *opts;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ctx;
    return TMC_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
  ctx->tune = tmc::Tuning::defaults(ctx->sms);
  {
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    ctx->priority = std::min(least, std::max(greatest, (int)ctx->opts.priority));
  }
  if (cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, ctx->priority) != cudaSuccess) {
    delete ctx;
    return TMC_ERR_CUDA;
  }
  // keep freed blocks pooled on the device between calls
  if (cudaDeviceGetDefaultMemPool(&ctx->pool, device) == cudaSuccess) {
    uint64_t thr = ctx->opts.reserve_bytes ? (uint64_t)ctx->opts.reserve_bytes : UINT64_MAX;
    cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (cudaMalloc(&ctx->d_stats, 8 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_pinned, 4096) != cudaSuccess) {
    tmc_ctx_destroy(ctx);
    return TMC_ERR_OOM;
  }
  *out = ctx;
  return TMC_OK;
}

tmc_status tmc_ctx_destroy(tmc_ctx* ctx) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) tmc::host_wait(ctx->stream);
  if (ctx->d_stats) cudaFree(ctx->d_stats);
  ctx->pinned.reset();  // the last context using the pool frees its blocks
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->copy_stream) {
    tmc::host_wait(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  if (ctx->copy_event) cudaEventDestroy(ctx->copy_event);
  for (cudaEvent_t e : ctx->slab_events) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return TMC_OK;
}

const char* tmc_last_error(const tmc_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }
void* tmc_ctx_stream(tmc_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
int64_t tmc_ctx_launch_count(const tmc_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }

tmc_status tmc_ctx_synchronize(tmc_ctx* ctx) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  TMC_CUDA(ctx, tmc::host_wait(ctx->stream));
  return TMC_OK;
}

tmc_status tmc_ctx_set_profiling(tmc_ctx* ctx, int on) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  TMC_CUDA(ctx, tmc::host_wait(ctx->stream));
  ctx->prof.collect();
  ctx->prof.on = on != 0;
  ctx->prof.acc.clear();
  return TMC_OK;
}

tmc_status tmc_ctx_set_tuning(tmc_ctx* ctx, int32_t key, int64_t value) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  switch (key) {
    case TMC_TUNE_GROUP_LANES:
      if (value < 0) break;
      ctx->tune.group_lanes = value;
      return TMC_OK;
    case TMC_TUNE_WARP_LIST_MAX:
      if (value < 0 || value > 0x7fffffff) break;
      ctx->tune.warp_list_max = value;
      return TMC_OK;
    case TMC_TUNE_VERTEX_BLOCKS_PER_SM:
      if (value < 1 || value > 64) break;
      ctx->tune.vertex_blocks_per_sm = (int)value;
      return TMC_OK;
    case TMC_TUNE_EMIT_BLOCKS_PER_SM:
      if (value < 1 || value > 64) break;
      ctx->tune.emit_blocks_per_sm = (int)value;
      return TMC_OK;
    case TMC_TUNE_SLAB_MIB:
      if (value < 4 || value > 1024) break;
      ctx->tune.slab_bytes = value << 20;
      return TMC_OK;
    case TMC_TUNE_MAX_SLABS:
      if (value < 2 || value > 64) break;
      ctx->tune.max_slabs = (int)value;
      return TMC_OK;
    case TMC_TUNE_QUAD_BLOCKS_PER_SM:
      if (value < 1 || value > 64) break;
      ctx->tune.quad_blocks_per_sm = (int)value;
      return TMC_OK;
    default:
      return fail(ctx, TMC_ERR_INVALID_ARG, "unknown tuning key %d", key);
  }
  return fail(ctx, TMC_ERR_INVALID_ARG, "tuning key %d: value %lld out of range", key, (long long)value);
}

tmc_status tmc_ctx_get_tuning(const tmc_ctx* ctx, int32_t key, int64_t* value) {
  if (!ctx || !value) return TMC_ERR_INVALID_ARG;
  switch (key) {
    case TMC_TUNE_GROUP_LANES: *value = ctx->tune.group_lanes; return TMC_OK;
    case TMC_TUNE_WARP_LIST_MAX: *value = ctx->tune.warp_list_max; return TMC_OK;
    case TMC_TUNE_VERTEX_BLOCKS_PER_SM: *value = ctx->tune.vertex_blocks_per_sm; return TMC_OK;
    case TMC_TUNE_EMIT_BLOCKS_PER_SM: *value = ctx->tune.emit_blocks_per_sm; return TMC_OK;
    case TMC_TUNE_SLAB_MIB: *value = ctx->tune.slab_bytes >> 20; return TMC_OK;
    case TMC_TUNE_MAX_SLABS: *value = ctx->tune.max_slabs; return TMC_OK;
    case TMC_TUNE_QUAD_BLOCKS_PER_SM: *value = ctx->tune.quad_blocks_per_sm; return TMC_OK;
    default: return TMC_ERR_INVALID_ARG;
  }
}

int32_t tmc_ctx_profile_read(tmc_ctx* ctx, int32_t max, char* names, double* ms, int64_t* counts) {
  if (!ctx) return -1;
  if (tmc::host_wait(ctx->stream) != cudaSuccess) return -1;
  ctx->prof.collect();
  int32_t i = 0;
  for (auto& kv : ctx->prof.acc) {
    if (i >= max) break;
    if (names) {
      std::strncpy(names + 32 * i, kv.first.c_str(), 31);
      names[32 * i + 31] = 0;
    }
    if (ms) ms[i] = kv.second.first;
    if (counts) counts[i] = kv.second.second;
    i++;
  }
  return i;
}

tmc_status tmc_mesh_free(tmc_ctx* ctx, tmc_mesh* mesh) {
  if (!ctx || !mesh) return TMC_ERR_INVALID_ARG;
  MeshPriv* mp = (MeshPriv*)mesh->priv;
  if (mp) {
    cudaSetDevice(ctx->device);
    for (void* p : mp->dev) cudaFreeAsync(p, ctx->stream);
    mp->shared.reset();
    tmc::host_wait(ctx->stream);  // the next call may reuse these pinned blocks
    for (void* p : mp->host) ctx->pinned_put(p);
    delete mp;
  }
  mesh_reset(mesh);
  return TMC_OK;
}

tmc_status tmc_dmc_extract(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out) {
  return dmc_extract(ctx, vol, iso, flags, out, nullptr);
}

tmc_status tmc_dmc_extract_generated(tmc_ctx* ctx, const tmc_generator* gen, double iso, uint32_t flags,
                                                tmc_mesh* out) {
  if (!ctx || !out) return fail(ctx, TMC_ERR_INVALID_ARG, "context or output is NULL");
  mesh_reset(out);
  FusedGen fg;
  tmc_volume vol;
  if (tmc_status s = gen_volume(ctx, gen, fg, vol)) return s;
  return dmc_extract(ctx, &vol, iso, flags, out, &fg);
}

// colorFaces + vertexValence as a stage of their own (cpp_dmc/DualMarchingCubes.cpp:714-871): the
// P3X3Y colour pass of tmc_dmc_extract runs the same code on its front-end mesh.
tmc_status tmc_dmc_color_valence(tmc_ctx* ctx, int64_t nr_v, int64_t nr_q, const int32_t* quads, uint8_t* colors,
                                 int32_t* valence) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  if (nr_v < 0 || nr_q < 0 || nr_v > INT32_MAX || 4 * nr_q > INT32_MAX)
    return fail(ctx, TMC_ERR_INVALID_ARG, "vertex or quad count out of range");
  if ((nr_q > 0 && (!quads || !colors)) || (nr_v > 0 && !valence))
    return fail(ctx, TMC_ERR_INVALID_ARG, "quads, colors or valence is NULL");
  TMC_CUDA(ctx, cudaSetDevice(ctx->device));
  const tmc::DmcPostStatus ps = tmc::dmc_color_valence(quads, nr_q, nr_v, colors, valence, ctx->sms, ctx->stream);
  ctx->launches += ps.launches;
  TMC_CUDA(ctx, ps.err);
  TMC_CUDA(ctx, tmc::host_wait(ctx->stream));
  return TMC_OK;
}

}  // extern "C"

namespace {

tmc_status dmc_extract(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out,
                       const FusedGen* fg) {
  if (!ctx || !out) return fail(ctx, TMC_ERR_INVALID_ARG, "context or output is NULL");
  mesh_reset(out);
  tmc_status s = fg ? TMC_OK : check_volume(ctx, vol);
  if (s) return s;
  if (!std::isfinite(iso)) return fail(ctx, TMC_ERR_INVALID_ARG, "isovalue must be finite");
  if (flags & TMC_DMC_SIMPLIFY) flags |= TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333;
  const bool simplify = flags & (TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333);
  if ((flags & TMC_OUT_LOCAL) && simplify)
    return fail(ctx, TMC_ERR_INVALID_ARG, "local coordinates exist only without simplification");
  TMC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  Allocs al(ctx);
  const float* field = nullptr;
  std::vector<tmc::TileGate> gates;
  tmc::GenParams* dev_params = nullptr;
  if ((s = fg ? fused_field(ctx, vol, *fg, al, &field, &dev_params) : field_slabs(ctx, vol, al, &field, gates)))
    return s;
  tmc::Grid g = make_grid(vol, field, iso);
  if (fg) set_fused(g, *fg, dev_params);
  g.flags = ((flags & TMC_GRAD_FLIP) ? tmc::kGridFlip : 0) | (simplify ? tmc::kGridNormal64 : 0);
  const tmc::CellSpace space = tmc::single_space(g);
  const int64_t ncell = g.ncells();

  tmc::DmcScratch sc{};
  TMC_CUDA(ctx, al.get(&sc.rec, ncell));
  TMC_CUDA(ctx, al.get(&sc.voff, ncell));
  TMC_CUDA(ctx, al.get(&sc.qoff, ncell));
  TMC_CUDA(ctx, al.get(&sc.cellof, ncell));
  TMC_CUDA(ctx, al.get(&sc.ccase, ncell));
  TMC_CUDA(ctx, al.get(&sc.amb_n, 1));
  TMC_CUDA(ctx, al.get(&sc.mask, tmc::dmc_tiles(space) * (tmc::kScanTile / 32)));
  TMC_CUDA(ctx, al.get(&sc.tile_sums, tmc::dmc_tiles(space)));
  TMC_CUDA(ctx, al.get(&sc.totals, 2));
  sc.stats = ctx->d_stats;
  TMC_CUDA(ctx, cudaMemsetAsync(sc.stats, 0, 8 * sizeof(unsigned long long), st));
  ctx->launches += tmc::dmc_front_count(space, sc, st, &ctx->prof, gates.data(), (int)gates.size());
  unsigned long long* h = (unsigned long long*)ctx->h_pinned;
  TMC_CUDA(ctx, cudaMemcpyAsync(h, sc.totals, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, tmc::host_wait(st));
  const int64_t nv = (int64_t)(h[0] >> 32), nq = (int64_t)(h[0] & 0xffffffffull);

  MeshPriv* mp = new (std::nothrow) MeshPriv();
  if (!mp) return fail(ctx, TMC_ERR_OOM, "host allocation failed");
  auto own = [&](void* p) {
    al.release(p);
    mp->dev.push_back(p);
  };
  tmc::DmcVertexOut vo{};
  int32_t* quads = nullptr;
  uint8_t* colors = nullptr;
  cudaError_t ce = cudaSuccess;
#define TMC_GET(ptr, count)                 \
  do {                                      \
    ce = al.get(&(ptr), (count));           \
    if (ce != cudaSuccess) {                \
      delete mp;                            \
      TMC_CUDA(ctx, ce);                    \
    }                                       \
    own(ptr);                               \
  } while (0)
  TMC_GET(vo.v, 3 * nv);
  TMC_GET(vo.n, 3 * nv);
  // simplification and the triangle split work on float64 positions, as the reference does
  const bool need_f64 = (flags & (TMC_OUT_POS_F64 | TMC_OUT_TRIANGLES)) || simplify;
  if (need_f64) TMC_GET(vo.v64, 3 * nv);
  if (simplify) TMC_GET(vo.n64, 3 * nv);
  if (flags & TMC_OUT_LOCAL) {
    TMC_GET(vo.vcell, nv);
    TMC_GET(vo.vuvw, 3 * nv);
  }
  TMC_GET(quads, 4 * nq);
  ce = al.get(&colors, nq);
  if (ce != cudaSuccess) {
    delete mp;
    TMC_CUDA(ctx, ce);
  }
  ce = al.get(&sc.vwork, nv);
  if (ce == cudaSuccess) ce = al.get(&sc.vrank, nv);
  if (ce == cudaSuccess) ce = dmc_vertex_scratch(al, sc, nv);
  if (ce != cudaSuccess) {
    delete mp;
    TMC_CUDA(ctx, ce);
  }
  ctx->launches += tmc::dmc_front_emit(space, sc, vo, nv, quads, colors, (flags & TMC_GRAD_FLIP) ? 1 : 0, ctx->tune, st,
                                       &ctx->prof);
  TMC_CUDA(ctx, cudaGetLastError());

  tmc::DmcMesh mesh{};
  mesh.nv = nv;
  mesh.nq = nq;
  mesh.v = vo.v;
  mesh.n = vo.n;
  mesh.v64 = vo.v64;
  mesh.n64 = vo.n64;
  mesh.quads = quads;
  mesh.colors = colors;
  tmc::DmcPostOut post{};
  EarlyCopies early{ctx, mp};
  const tmc::ReadyFn ready = [&early](const void* dev, size_t bytes) { early.issue(dev, bytes); };
  tmc::DmcPostStatus ps =
      tmc::dmc_postprocess(mesh, flags, ctx->sms, st, &post, (unsigned long long*)ctx->h_pinned + 64, &ctx->prof,
                           false, (flags & TMC_OUT_HOST) ? &ready : nullptr);
  if (ps.err == cudaSuccess) ps.err = early.err;
  if (ps.err != cudaSuccess) {
    if (ctx->copy_stream) tmc::host_wait(ctx->copy_stream);
    for (void* p : mp->host) ctx->pinned_put(p);
    delete mp;
    TMC_CUDA(ctx, ps.err);
  }
  ctx->launches += ps.launches;
  for (void* p : post.owned) mp->dev.push_back(p);
  for (void* p : post.freed) {
    al.release(p);
    for (auto& q : mp->dev)
      if (q == p) q = nullptr;
  }
  {
    std::vector<void*> keep;
    for (void* q : mp->dev)
      if (q) keep.push_back(q);
    mp->dev.swap(keep);
  }
  out->nr_v = post.mesh.nv;
  out->nr_q = post.mesh.nq;
  out->v = post.mesh.v;
  out->n = post.mesh.n;
  out->v64 = post.mesh.v64;
  // internal float64 buffers that are not outputs
  auto drop = [&](void* ptr) {
    if (!ptr) return;
    for (auto& q : mp->dev)
      if (q == ptr) q = nullptr;
    std::vector<void*> keep;
    for (void* q : mp->dev)
      if (q) keep.push_back(q);
    mp->dev.swap(keep);
    cudaFreeAsync(ptr, st);
  };
  if (out->v64 && !(flags & TMC_OUT_POS_F64)) {
    drop(out->v64);
    out->v64 = nullptr;
  }
  drop(post.mesh.n64);
  out->quads = post.mesh.quads;
  out->nr_t = post.nt;
  out->tris = post.tris;
  out->nr_he = post.nhe;
  out->he = post.he;
  out->he_v = post.he_v;
  out->he_f = post.he_f;
  out->vcell = vo.vcell;
  out->vuvw = vo.vuvw;
  TMC_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, tmc::host_wait(st));
  for (int q = 0; q < 8; q++) out->stats[q] = (int64_t)h[q];
  ctx->prof.collect();
  out->stats[4] = post.non_manifold;
  out->stats[6] = ncell;
#undef TMC_GET
  return finish_mesh(ctx, flags, out, mp, &early);
}

// TMC extraction driver shared by the shared-vertex and halfedge entry points.
tmc_status tmc_extract(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out, bool halfedge,
                       const FusedGen* fg = nullptr) {
  if (!ctx || !out) return fail(ctx, TMC_ERR_INVALID_ARG, "context or output is NULL");
  mesh_reset(out);
  tmc_status s = fg ? TMC_OK : check_volume(ctx, vol);
  if (s) return s;
  if (!std::isfinite(iso)) return fail(ctx, TMC_ERR_INVALID_ARG, "isovalue must be finite");
  if (flags & (TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333 | TMC_OUT_LOCAL))
    return fail(ctx, TMC_ERR_INVALID_ARG, "DMC-only flag given to a TMC extraction");
  if (halfedge) flags |= TMC_OUT_HALFEDGES;
  TMC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  Allocs al(ctx);
  const float* field = nullptr;
  std::vector<tmc::TileGate> gates;
  tmc::GenParams* dev_params = nullptr;
  if ((s = fg ? fused_field(ctx, vol, *fg, al, &field, &dev_params) : field_slabs(ctx, vol, al, &field, gates)))
    return s;
  tmc::Grid g = make_grid(vol, field, iso);
  if (fg) set_fused(g, *fg, dev_params);
  g.flags = (flags & TMC_OUT_POS_F64) ? tmc::kGridPos64 : 0;
  const int64_t ncell = g.ncells();
  tmc::TmcScratch sc{};
  TMC_CUDA(ctx, al.get(&sc.rec, ncell));
  TMC_CUDA(ctx, al.get(&sc.voff, ncell));
  TMC_CUDA(ctx, al.get(&sc.toff, ncell));
  TMC_CUDA(ctx, al.get(&sc.cellof, ncell));
  const tmc::CellSpace space = tmc::single_space(g);
  TMC_CUDA(ctx, al.get(&sc.mask, tmc::tmc_tiles(space) * (tmc::kScanTile / 32)));
  TMC_CUDA(ctx, al.get(&sc.tile_sums, tmc::tmc_tiles(space)));
  TMC_CUDA(ctx, al.get(&sc.totals, 2));
  TMC_CUDA(ctx, al.get(&sc.amb_n, 1));
  sc.stats = ctx->d_stats;
  TMC_CUDA(ctx, cudaMemsetAsync(sc.stats, 0, 8 * sizeof(unsigned long long), st));
  ctx->launches += tmc::tmc_classify(space, sc, st, &ctx->prof, gates.data(), (int)gates.size());
  unsigned long long* h = (unsigned long long*)ctx->h_pinned;
  int64_t n_amb = 0;
  TMC_CUDA(ctx, tmc_ambiguous_records(ctx, al, sc, n_amb));
  ctx->launches += tmc::tmc_count(space, sc, n_amb, ctx->sms, st, &ctx->prof);
  TMC_CUDA(ctx, cudaMemcpyAsync(h, sc.totals, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, cudaMemcpyAsync(h + 1, sc.stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, tmc::host_wait(st));
  const int64_t nv = (int64_t)(h[0] >> 32), nt = (int64_t)(h[0] & 0xffffffffull);

  MeshPriv* mp = new (std::nothrow) MeshPriv();
  if (!mp) return fail(ctx, TMC_ERR_OOM, "host allocation failed");
  cudaError_t ce = cudaSuccess;
#define TMC_OWN(ptr, count)                 \
  do {                                      \
    ce = al.get(&(ptr), (count));           \
    if (ce != cudaSuccess) {                \
      delete mp;                            \
      TMC_CUDA(ctx, ce);                    \
    }                                       \
    al.release(ptr);                        \
    mp->dev.push_back(ptr);                 \
  } while (0)
  tmc::TmcVertexOut vo{};
  int32_t* tris = nullptr;
  TMC_OWN(vo.v, 3 * nv);
  TMC_OWN(vo.n, 3 * nv);
  if (flags & TMC_OUT_POS_F64) TMC_OWN(vo.v64, 3 * nv);
  TMC_OWN(tris, 3 * nt);
  ctx->launches += tmc::tmc_emit(space, sc, n_amb, vo, tris, ctx->tune, st, &ctx->prof);
  TMC_CUDA(ctx, cudaGetLastError());
  out->nr_v = nv;
  out->nr_t = nt;
  out->v = vo.v;
  out->n = vo.n;
  out->v64 = vo.v64;
  out->tris = tris;
  int64_t non_manifold = 0;
  EarlyCopies early{ctx, mp};
  if ((flags & TMC_OUT_HOST) && (flags & TMC_OUT_HALFEDGES)) {
    // the vertices and triangles are final: copy them out while the halfedges are built
    early.issue(vo.v, (size_t)nv * 3 * sizeof(float));
    early.issue(vo.n, (size_t)nv * 3 * sizeof(float));
    early.issue(vo.v64, (size_t)nv * 3 * sizeof(double));
    early.issue(tris, (size_t)nt * 3 * sizeof(int32_t));
    if (early.err != cudaSuccess) {
      if (ctx->copy_stream) tmc::host_wait(ctx->copy_stream);
      for (void* p : mp->host) ctx->pinned_put(p);
      delete mp;
      TMC_CUDA(ctx, early.err);
    }
  }
  if (flags & TMC_OUT_HALFEDGES) {
    const int64_t nh = 3 * nt;
    int32_t *twin = nullptr, *he4 = nullptr, *hv = nullptr, *hf = nullptr;
    uint8_t* flag = nullptr;
    tmc::HeWork w{};
    TMC_CUDA(ctx, al.get(&w.deg, nv));
    TMC_CUDA(ctx, al.get(&w.off, nv));
    TMC_CUDA(ctx, al.get(&w.rank, nh));
    TMC_CUDA(ctx, al.get(&w.list, nh));
    TMC_CUDA(ctx, al.get(&w.hv_key, nv));
    TMC_CUDA(ctx, al.get(&w.tiles, tmc::scan_tiles(nv) + 2));
    TMC_CUDA(ctx, al.get(&w.total, 2));
    TMC_CUDA(ctx, al.get(&w.non_manifold, 2));
    TMC_CUDA(ctx, al.get(&twin, nh));
    TMC_CUDA(ctx, al.get(&flag, nh));
    TMC_CUDA(ctx, cudaMemsetAsync(w.non_manifold, 0, 2 * sizeof(unsigned long long), st));
    TMC_OWN(he4, 4 * nh);
    TMC_OWN(hv, nv);
    TMC_OWN(hf, nt);
    tmc::HeOut ho{twin, flag, hv};
    tmc::Stage stage(&ctx->prof, "tmc_halfedges", st);
    ctx->launches += tmc::build_halfedges(tris, 3, nt, nv, ho, w, ctx->sms, st);
    ctx->launches += tmc::pack_halfedges4(tris, 3, twin, nh, he4, hf, ctx->sms, st);
    TMC_CUDA(ctx, cudaGetLastError());
    TMC_CUDA(ctx, cudaMemcpyAsync(h + 8, w.non_manifold, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    TMC_CUDA(ctx, tmc::host_wait(st));
    non_manifold = (int64_t)h[8];
    out->nr_he = nh;
    out->he = he4;
    out->he_v = hv;
    out->he_f = hf;
  }
#undef TMC_OWN
  TMC_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, tmc::host_wait(st));
  for (int q = 0; q < 8; q++) out->stats[q] = (int64_t)h[q];
  ctx->prof.collect();
  out->stats[4] = non_manifold;
  out->stats[6] = ncell;
  return finish_mesh(ctx, flags, out, mp, &early);
}

// One batch of requests of one algorithm: all volumes share one cell space, so every stage is one
// launch for the whole batch; one host synchronisation reads the per-volume output sizes.
// Requests with simplification, triangles or halfedges finish with the per-mesh post-processing on
// their slice of the batch's arrays.
tmc_status batch_run(tmc_ctx* ctx, const std::vector<int>& idx, const tmc_request* reqs, tmc_mesh* outs, bool dmc) {
  const int nb = (int)idx.size();
  tmc_status s = TMC_OK;
  bool any_f64 = false, any_n64 = false, any_local = false, any_amb = false;
  for (int q = 0; q < nb; q++) {
    const tmc_request& r = reqs[idx[q]];
    if ((s = check_volume(ctx, &r.vol))) return fail(ctx, s, "request %d: %s", idx[q], ctx->err.c_str());
    if (!std::isfinite(r.iso)) return fail(ctx, TMC_ERR_INVALID_ARG, "request %d: isovalue must be finite", idx[q]);
    uint32_t f = r.flags;
    if (f & TMC_DMC_SIMPLIFY) f |= TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333;
    const bool simp = f & (TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333);
    if (dmc) {
      if ((f & TMC_OUT_LOCAL) && simp)
        return fail(ctx, TMC_ERR_INVALID_ARG, "request %d: local coordinates exist only without simplification",
                    idx[q]);
      any_f64 |= (f & (TMC_OUT_POS_F64 | TMC_OUT_TRIANGLES)) || simp;
      any_n64 |= simp;
      any_local |= (f & TMC_OUT_LOCAL) != 0;
    } else {
      if (f & (TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333 | TMC_OUT_LOCAL))
        return fail(ctx, TMC_ERR_INVALID_ARG, "request %d: DMC-only flag given to a TMC extraction", idx[q]);
      any_f64 |= (f & TMC_OUT_POS_F64) != 0;
    }
  }
  TMC_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  Allocs al(ctx);
  // ---- the cell space: volumes one after another, each from a tile boundary ----
  std::vector<tmc::Grid> grids(nb);
  std::vector<int64_t> tile0(nb + 1, 0);
  for (int q = 0; q < nb; q++) {
    const tmc_request& r = reqs[idx[q]];
    const float* field = nullptr;
    if ((s = field_on_device(ctx, &r.vol, al, &field))) return s;
    grids[q] = make_grid(&r.vol, field, r.iso);
    {
      const bool simp = r.flags & (TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333);
      grids[q].flags = dmc ? (((r.flags & TMC_GRAD_FLIP) ? tmc::kGridFlip : 0) | (simp ? tmc::kGridNormal64 : 0))
                           : ((r.flags & TMC_OUT_POS_F64) ? tmc::kGridPos64 : 0);
    }
    grids[q].vbase = tile0[q] * tmc::kScanTile;
    tile0[q + 1] = tile0[q] + tmc::ceil_div(grids[q].ncells(), tmc::kScanTile);
  }
  const int64_t tiles = tile0[nb];
  const int64_t ncell = tiles * tmc::kScanTile;
  if (ncell > ((int64_t)1 << 32) - tmc::kScanTile)
    return fail(ctx, TMC_ERR_CAPACITY, "batch of %lld cells: a batch holds at most 2^32 cells", (long long)ncell);
  std::vector<int32_t> tile_vol((size_t)tiles);
  for (int q = 0; q < nb; q++)
    for (int64_t t = tile0[q]; t < tile0[q + 1]; t++) tile_vol[(size_t)t] = q;
  tmc::Grid* d_grids = nullptr;
  int32_t* d_tile_vol = nullptr;
  TMC_CUDA(ctx, al.get(&d_grids, nb));
  TMC_CUDA(ctx, al.get(&d_tile_vol, tiles));
  TMC_CUDA(ctx, cudaMemcpyAsync(d_grids, grids.data(), nb * sizeof(tmc::Grid), cudaMemcpyHostToDevice, st));
  TMC_CUDA(ctx, cudaMemcpyAsync(d_tile_vol, tile_vol.data(), tiles * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  tmc::CellSpace space{};
  space.one = grids[0];
  space.grids = d_grids;
  space.tile_vol = d_tile_vol;
  space.n = ncell;

  // ---- count ----
  uint32_t* rec = nullptr;
  int32_t *voff = nullptr, *qoff = nullptr;
  unsigned long long *tile_sums = nullptr, *totals = nullptr;
  tmc::CellMask* mask = nullptr;
  uint16_t* cellof = nullptr;
  TMC_CUDA(ctx, al.get(&rec, ncell));
  TMC_CUDA(ctx, al.get(&voff, ncell));
  TMC_CUDA(ctx, al.get(&qoff, ncell));
  TMC_CUDA(ctx, al.get(&cellof, ncell));
  TMC_CUDA(ctx, al.get(&mask, tiles * (tmc::kScanTile / 32)));
  TMC_CUDA(ctx, al.get(&tile_sums, tiles));
  TMC_CUDA(ctx, al.get(&totals, 2));
  TMC_CUDA(ctx, cudaMemsetAsync(ctx->d_stats, 0, 8 * sizeof(unsigned long long), st));
  tmc::DmcScratch dsc{};
  tmc::TmcScratch tsc{};
  int64_t n_amb_rec = 0;
  if (dmc) {
    dsc = tmc::DmcScratch{rec, voff, qoff, nullptr, tile_sums, totals, ctx->d_stats};
    dsc.mask = mask;
    dsc.cellof = cellof;
    TMC_CUDA(ctx, al.get(&dsc.amb_n, 1));
    TMC_CUDA(ctx, al.get(&dsc.ccase, ncell));
    ctx->launches += tmc::dmc_front_count(space, dsc, st, &ctx->prof);
  } else {
    tsc = tmc::TmcScratch{rec, voff, qoff, tile_sums, totals, ctx->d_stats};
    tsc.mask = mask;
    tsc.cellof = cellof;
    TMC_CUDA(ctx, al.get(&tsc.amb_n, 1));
    ctx->launches += tmc::tmc_classify(space, tsc, st, &ctx->prof);
    TMC_CUDA(ctx, tmc_ambiguous_records(ctx, al, tsc, n_amb_rec));
    ctx->launches += tmc::tmc_count(space, tsc, n_amb_rec, ctx->sms, st, &ctx->prof);
  }
  std::vector<unsigned long long> toff((size_t)tiles + 1);
  unsigned long long* h = (unsigned long long*)ctx->h_pinned;
  TMC_CUDA(ctx, cudaMemcpyAsync(toff.data(), tile_sums, tiles * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, cudaMemcpyAsync(h, totals, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, cudaMemcpyAsync(h + 1, ctx->d_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  TMC_CUDA(ctx, tmc::host_wait(st));
  toff[(size_t)tiles] = h[0];
  const int64_t NV = (int64_t)(h[0] >> 32), NF = (int64_t)(h[0] & 0xffffffffull);
  if (NV >= ((int64_t)1 << 31) || NF >= ((int64_t)1 << 31))
    return fail(ctx, TMC_ERR_CAPACITY, "batch output above 2^31 vertices or faces; split the batch");
  std::vector<int64_t> vb(nb + 1), fb(nb + 1);
  for (int q = 0; q <= nb; q++) {
    const unsigned long long w = toff[(size_t)tile0[q]];
    vb[q] = (int64_t)(w >> 32);
    fb[q] = (int64_t)(w & 0xffffffffull);
  }

  // ---- outputs shared by the batch's meshes ----
  auto block = std::make_shared<SharedBlock>();
  block->stream = st;
  cudaError_t ce = cudaSuccess;
  auto get_shared = [&](auto** p, int64_t count) -> cudaError_t {
    ce = al.get(p, count);
    if (ce == cudaSuccess) {
      al.release(*p);
      block->dev.push_back(*p);
    }
    return ce;
  };
  float *v = nullptr, *nn = nullptr, *vuvw = nullptr;
  double *v64 = nullptr, *n64 = nullptr;
  int64_t* vcell = nullptr;
  int32_t* faces = nullptr;
  uint8_t* colors = nullptr;
  TMC_CUDA(ctx, get_shared(&v, 3 * NV));
  TMC_CUDA(ctx, get_shared(&nn, 3 * NV));
  if (any_f64) TMC_CUDA(ctx, get_shared(&v64, 3 * NV));
  if (dmc) {
    if (any_n64) TMC_CUDA(ctx, get_shared(&n64, 3 * NV));
    if (any_local) {
      TMC_CUDA(ctx, get_shared(&vcell, NV));
      TMC_CUDA(ctx, get_shared(&vuvw, 3 * NV));
    }
    TMC_CUDA(ctx, get_shared(&faces, 4 * NF));
    TMC_CUDA(ctx, get_shared(&colors, NF));
    TMC_CUDA(ctx, al.get(&dsc.vwork, NV));
    TMC_CUDA(ctx, al.get(&dsc.vrank, NV));
    TMC_CUDA(ctx, dmc_vertex_scratch(al, dsc, NV));
    tmc::DmcVertexOut vo{v, nn, v64, n64, vcell, vuvw};
    ctx->launches += tmc::dmc_front_emit(space, dsc, vo, NV, faces, colors, 0, ctx->tune, st, &ctx->prof);
  } else {
    TMC_CUDA(ctx, get_shared(&faces, 3 * NF));
    tmc::TmcVertexOut vo{v, nn, v64};
    ctx->launches += tmc::tmc_emit(space, tsc, n_amb_rec, vo, faces, ctx->tune, st, &ctx->prof);
  }
  TMC_CUDA(ctx, cudaGetLastError());

  // ---- one mesh per request ----
  for (int q = 0; q < nb; q++) {
    const tmc_request& r = reqs[idx[q]];
    tmc_mesh* out = &outs[idx[q]];
    uint32_t f = r.flags;
    if (f & TMC_DMC_SIMPLIFY) f |= TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333;
    const bool simp = dmc && (f & (TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333));
    const int64_t nv = vb[q + 1] - vb[q], nf = fb[q + 1] - fb[q];
    MeshPriv* mp = new (std::nothrow) MeshPriv();
    if (!mp) return fail(ctx, TMC_ERR_OOM, "host allocation failed");
    mp->shared = block;
    out->priv = mp;
    out->stats[6] = grids[q].ncells();
    float* sv = v + 3 * vb[q];
    float* sn = nn + 3 * vb[q];
    double* sv64 = v64 ? v64 + 3 * vb[q] : nullptr;
    if (dmc) {
      tmc::DmcMesh mesh{};
      mesh.nv = nv;
      mesh.nq = nf;
      mesh.v = sv;
      mesh.n = sn;
      mesh.v64 = sv64;
      mesh.n64 = n64 ? n64 + 3 * vb[q] : nullptr;
      mesh.quads = faces + 4 * fb[q];
      mesh.colors = colors + fb[q];
      tmc::DmcPostOut post{};
      if (simp || (f & (TMC_OUT_TRIANGLES | TMC_OUT_HALFEDGES))) {
        tmc::DmcPostStatus ps = tmc::dmc_postprocess(mesh, f, ctx->sms, st, &post,
                                                     (unsigned long long*)ctx->h_pinned + 64, &ctx->prof, true);
        for (void* p : post.owned) mp->dev.push_back(p);
        if (ps.err != cudaSuccess) TMC_CUDA(ctx, ps.err);
        ctx->launches += ps.launches;
      } else {
        post.mesh = mesh;
      }
      out->nr_v = post.mesh.nv;
      out->nr_q = post.mesh.nq;
      out->v = post.mesh.v;
      out->n = post.mesh.n;
      out->v64 = (f & TMC_OUT_POS_F64) ? post.mesh.v64 : nullptr;
      out->quads = post.mesh.quads;
      out->nr_t = post.nt;
      out->tris = post.tris;
      out->nr_he = post.nhe;
      out->he = post.he;
      out->he_v = post.he_v;
      out->he_f = post.he_f;
      if (f & TMC_OUT_LOCAL) {
        out->vcell = vcell + vb[q];
        out->vuvw = vuvw + 3 * vb[q];
      }
      out->stats[4] = post.non_manifold;
      // float64 arrays the post-processing made that are not outputs
      auto drop = [&](void* ptr) {
        if (!ptr) return;
        for (auto& d : mp->dev)
          if (d == ptr) {
            d = nullptr;
            cudaFreeAsync(ptr, st);
          }
      };
      if (!(f & TMC_OUT_POS_F64)) drop(post.mesh.v64);
      drop(post.mesh.n64);
      std::vector<void*> keep;
      for (void* d : mp->dev)
        if (d) keep.push_back(d);
      mp->dev.swap(keep);
    } else {
      out->nr_v = nv;
      out->nr_t = nf;
      out->v = sv;
      out->n = sn;
      out->v64 = (f & TMC_OUT_POS_F64) ? sv64 : nullptr;
      out->tris = faces + 3 * fb[q];
      if (f & TMC_OUT_HALFEDGES) {
        const int64_t nh = 3 * nf;
        int32_t *twin = nullptr, *he4 = nullptr, *hv = nullptr, *hf = nullptr;
        uint8_t* flag = nullptr;
        tmc::HeWork w{};
        TMC_CUDA(ctx, al.get(&w.deg, nv));
        TMC_CUDA(ctx, al.get(&w.off, nv));
        TMC_CUDA(ctx, al.get(&w.rank, nh));
        TMC_CUDA(ctx, al.get(&w.list, nh));
        TMC_CUDA(ctx, al.get(&w.hv_key, nv));
        TMC_CUDA(ctx, al.get(&w.tiles, tmc::scan_tiles(nv) + 2));
        TMC_CUDA(ctx, al.get(&w.total, 2));
        TMC_CUDA(ctx, al.get(&w.non_manifold, 2));
        TMC_CUDA(ctx, al.get(&twin, nh));
        TMC_CUDA(ctx, al.get(&flag, nh));
        TMC_CUDA(ctx, cudaMemsetAsync(w.non_manifold, 0, 2 * sizeof(unsigned long long), st));
        TMC_CUDA(ctx, al.get(&he4, 4 * nh));
        al.release(he4);
        mp->dev.push_back(he4);
        TMC_CUDA(ctx, al.get(&hv, nv));
        al.release(hv);
        mp->dev.push_back(hv);
        TMC_CUDA(ctx, al.get(&hf, nf));
        al.release(hf);
        mp->dev.push_back(hf);
        tmc::HeOut ho{twin, flag, hv};
        tmc::Stage stage(&ctx->prof, "tmc_halfedges", st);
        ctx->launches += tmc::build_halfedges(out->tris, 3, nf, nv, ho, w, ctx->sms, st);
        ctx->launches += tmc::pack_halfedges4(out->tris, 3, twin, nh, he4, hf, ctx->sms, st);
        TMC_CUDA(ctx, cudaGetLastError());
        TMC_CUDA(ctx, cudaMemcpyAsync(h + 8, w.non_manifold, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        TMC_CUDA(ctx, tmc::host_wait(st));
        out->stats[4] = (int64_t)h[8];
        out->nr_he = nh;
        out->he = he4;
        out->he_v = hv;
        out->he_f = hf;
      }
    }
    if ((s = finish_mesh(ctx, f, out, mp))) return s;
  }
  ctx->prof.collect();
  return TMC_OK;
}

}  // namespace

extern "C" {
tmc_status tmc_tmc_sharedvertex(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out) {
  return tmc_extract(ctx, vol, iso, flags, out, false);
}
tmc_status tmc_tmc_halfedge(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out) {
  return tmc_extract(ctx, vol, iso, flags, out, true);
}
tmc_status tmc_tmc_extract_generated(tmc_ctx* ctx, const tmc_generator* gen, double iso, uint32_t flags,
                                     int32_t halfedge, tmc_mesh* out) {
  if (!ctx || !out) return fail(ctx, TMC_ERR_INVALID_ARG, "context or output is NULL");
  mesh_reset(out);
  FusedGen fg;
  tmc_volume vol;
  if (tmc_status s = gen_volume(ctx, gen, fg, vol)) return s;
  return tmc_extract(ctx, &vol, iso, flags, out, halfedge != 0, &fg);
}
tmc_status tmc_batch_extract(tmc_ctx* ctx, int32_t n, const tmc_request* reqs, tmc_mesh* outs) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  if (n < 0 || (n > 0 && (!reqs || !outs))) return fail(ctx, TMC_ERR_INVALID_ARG, "bad request array");
  for (int32_t b = 0; b < n; b++) mesh_reset(&outs[b]);
  std::vector<int> dmc, tmcs;
  for (int32_t b = 0; b < n; b++) {
    if (reqs[b].algo == TMC_ALGO_DMC) dmc.push_back(b);
    else if (reqs[b].algo == TMC_ALGO_TMC) tmcs.push_back(b);
    else return fail(ctx, TMC_ERR_INVALID_ARG, "request %d: unknown algorithm %u", b, reqs[b].algo);
  }
  tmc_status s = TMC_OK;
  if (!dmc.empty()) s = batch_run(ctx, dmc, reqs, outs, true);
  if (!s && !tmcs.empty()) s = batch_run(ctx, tmcs, reqs, outs, false);
  if (s) {
    const std::string msg = ctx->err;
    for (int32_t b = 0; b < n; b++) tmc_mesh_free(ctx, &outs[b]);
    ctx->err = msg;
  }
  return s;
}
}

// Autotuner: coordinate descent over the launch-shape settings, each candidate timed with CUDA
// events over `rounds` batched extractions of the caller's requests (after one untimed call).  A
// candidate replaces the current value only when it is at least 2 % faster.  The meshes do not
// depend on the settings, so the search only changes speed.
extern "C" tmc_status tmc_ctx_autotune(tmc_ctx* ctx, int32_t n, const tmc_request* reqs, int32_t rounds,
                                       double* best_ms) {
  if (!ctx) return TMC_ERR_INVALID_ARG;
  if (n <= 0 || !reqs || rounds < 1) return fail(ctx, TMC_ERR_INVALID_ARG, "autotune needs requests and rounds >= 1");
  std::vector<tmc_mesh> outs((size_t)n);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  TMC_CUDA(ctx, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(ctx, TMC_ERR_CUDA, "cudaEventCreate failed");
  }
  auto run = [&](bool timed, double& ms) -> tmc_status {
    const int reps = timed ? rounds : 1;
    cudaEventRecord(e0, ctx->stream);
    for (int r = 0; r < reps; r++) {
      tmc_status st;
      if (n == 1) {  // one request: the single-volume entry point (slab pipeline for a host field)
        const tmc_request& q = reqs[0];
        if (q.algo == TMC_ALGO_DMC) st = tmc_dmc_extract(ctx, &q.vol, q.iso, q.flags, outs.data());
        else if (q.flags & TMC_OUT_HALFEDGES) st = tmc_tmc_halfedge(ctx, &q.vol, q.iso, q.flags, outs.data());
        else st = tmc_tmc_sharedvertex(ctx, &q.vol, q.iso, q.flags, outs.data());
      } else {
        st = tmc_batch_extract(ctx, n, reqs, outs.data());
      }
      if (st) return st;
      for (auto& m : outs) tmc_mesh_free(ctx, &m);
    }
    cudaEventRecord(e1, ctx->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) return fail(ctx, TMC_ERR_CUDA, "autotune timing failed");
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    ms = t / reps;
    return TMC_OK;
  };
  const int64_t sm = ctx->sms;
  struct Axis {
    int32_t key;
    std::vector<int64_t> values;
  };
  const bool host_field = n == 1 && !reqs[0].vol.on_device;
  std::vector<Axis> axes = {
      {TMC_TUNE_GROUP_LANES, {0, sm * 12 * 32, sm * 24 * 32, sm * 48 * 32}},
      {TMC_TUNE_WARP_LIST_MAX, {0, sm * 8, sm * 32, sm * 128}},
      {TMC_TUNE_VERTEX_BLOCKS_PER_SM, {8, 16, 32}},
      {TMC_TUNE_EMIT_BLOCKS_PER_SM, {4, 8, 16}},
      {TMC_TUNE_QUAD_BLOCKS_PER_SM, {1, 2, 4}},
  };
  if (host_field) {
    axes.push_back({TMC_TUNE_SLAB_MIB, {8, 16, 32, 64, 128}});
    axes.push_back({TMC_TUNE_MAX_SLABS, {4, 8, 16, 32}});
  }
  double best = 0, ms = 0;
  tmc_status st = run(false, ms);  // warm-up: pools, pinned blocks
  if (!st) st = run(true, best);
  for (const Axis& ax : axes) {
    if (st) break;
    int64_t keep = 0;
    tmc_ctx_get_tuning(ctx, ax.key, &keep);
    const int64_t start = keep;
    for (int64_t v : ax.values) {
      if (v == start) continue;
      tmc_ctx_set_tuning(ctx, ax.key, v);
      st = run(true, ms);
      if (st) break;
      if (ms < 0.98 * best) {
        best = ms;
        keep = v;
      }
    }
    tmc_ctx_set_tuning(ctx, ax.key, keep);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (best_ms) *best_ms = best;
  return TMC_OK;
}

// Context access for entry points defined in other translation units (ctx_access.h).
namespace tmc {
int ctx_device(const tmc_ctx* ctx) { return ctx->device; }
cudaStream_t ctx_stream(const tmc_ctx* ctx) { return ctx->stream; }
tmc_status ctx_fail(tmc_ctx* ctx, tmc_status s, const char* msg) { return fail(ctx, s, "%s", msg); }
void ctx_count_launches(tmc_ctx* ctx, int64_t n) { ctx->launches += n; }
void ctx_share_pinned(tmc_ctx* ctx, tmc_ctx* from) { ctx->pinned = from->pinned; }
}  // namespace tmc
