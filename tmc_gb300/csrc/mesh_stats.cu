// Mesh validation metrics: element quality and the vertex valence distribution, as the reference's
// CUDA DMC computes them for its meshes.
//
//   quality  (p_mc::EstimateElementQuality, dmc/EstimateElementQuality.cu:1-56, with the measures of
//            p_mc::ElementQuality, dmc/ElementQuality.h:69-93): per quad the smallest of
//            2 |e1 x e2| / (|e1|^2 + |e2|^2) over its four corners (e1, e2 the corner's two edges);
//            per triangle the mean ratio 2 sqrt(3) |e1 x e2| / (l0 + l1 + l2), 0 when an edge has
//            zero length.  Float32 on float32 positions, as the reference.
//   valence  (p_mc::VertexValence::vertexValence, dmc/VertexValence.cu:79-170): the number of
//            distinct undirected edges at each vertex, as a histogram over 0..99.  The reference
//            finds the distinct edges with a hash table; here each face edge contributes its two
//            end points to per-vertex neighbour lists (degree count, scan, scatter) and each vertex
//            counts the distinct entries of its list.  Valences above 99 (where the reference would
//            index past its histogram) are counted in the last bin.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/tmc_gb300.h"
#include "common.cuh"
#include "ctx_access.h"
#include "halfedges.h"
#include "scan.cuh"

namespace tmc {
namespace {

constexpr int kValenceBins = 100;

__device__ __forceinline__ float3 ld3(const float* v, int i) { return make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
// the reference's cross product component order (ElementQuality::cross)
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.z * b.y - a.y * b.z, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float norm2(float3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

// 2 |(b - a) x (c - a)| / (|b - a|^2 + |c - a|^2): the quality of corner a between neighbours b and c
__device__ __forceinline__ float corner_q(float3 a, float3 b, float3 c) {
  const float3 e1 = sub3(b, a), e2 = sub3(c, a);
  return 2 * sqrtf(norm2(cross3(e1, e2))) / (norm2(e1) + norm2(e2));
}

// summary[0] min, [1] max (as float bits: qualities are >= 0, so their bits order as unsigned
// integers), sum in a double.  lo / hi / s are a lane's contribution (neutral values for lanes
// without a face).
__device__ __forceinline__ void summarise(float lo, float hi, double s, unsigned* mn, unsigned* mx, double* sum) {
  // warp reduction first: one atomic per warp and quantity
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mn, __float_as_uint(lo));
    atomicMax(mx, __float_as_uint(hi));
    atomicAdd(sum, s);
  }
}

__global__ void quality_kernel(const float* v, const int32_t* faces, int P, int64_t nf, float* out, unsigned* mn,
                               unsigned* mx, double* sum) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // every lane runs the same number of turns, so that the warp reductions see all lanes
  const int64_t turns = (nf + stride - 1) / stride;
  for (int64_t t = 0; t < turns; t++) {
    const int64_t f = t * stride + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = f < nf;
    float q = 0;
    if (live) {
      if (P == 4) {
        const int4 c = reinterpret_cast<const int4*>(faces)[f];
        const float3 p0 = ld3(v, c.x), p1 = ld3(v, c.y), p2 = ld3(v, c.z), p3 = ld3(v, c.w);
        const float q0 = corner_q(p0, p1, p3), q1 = corner_q(p1, p2, p0);
        const float q2 = corner_q(p2, p3, p1), q3 = corner_q(p3, p0, p2);
        q = q0 < q1 ? q0 : q1;
        q = q < q2 ? q : q2;
        q = q < q3 ? q : q3;
      } else {
        const int32_t* c = faces + 3 * f;
        const float3 p0 = ld3(v, c[0]), p1 = ld3(v, c[1]), p2 = ld3(v, c[2]);
        const float a = sqrtf(norm2(cross3(sub3(p1, p0), sub3(p2, p0))));
        const float l0 = norm2(sub3(p1, p0)), l1 = norm2(sub3(p2, p1)), l2 = norm2(sub3(p0, p2));
        if (l0 != 0 && l1 != 0 && l2 != 0) q = 2 * sqrtf(3.0f) * a / (l0 + l1 + l2);
      }
      out[f] = q;
    }
    // lanes past the end add nothing: +inf to the min, 0 to the max and the sum
    summarise(live ? q : INFINITY, live ? q : 0.0f, live ? (double)q : 0.0, mn, mx, sum);
  }
}

// valence: neighbour entries per vertex (both ends of every face edge)
__global__ void nbr_count_kernel(const int32_t* faces, int P, int64_t nf, int32_t* cnt) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nf * P; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int a = faces[h], b = faces[f * P + (r + 1) % P];
    if (a == b) continue;
    atomicAdd(cnt + a, 1);
    atomicAdd(cnt + b, 1);
  }
}
__global__ void nbr_scatter_kernel(const int32_t* faces, int P, int64_t nf, const int32_t* off, int32_t* cursor,
                                   int32_t* nbr) {
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nf * P; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int a = faces[h], b = faces[f * P + (r + 1) % P];
    if (a == b) continue;
    nbr[off[a] + atomicAdd(cursor + a, 1)] = b;
    nbr[off[b] + atomicAdd(cursor + b, 1)] = a;
  }
}
// distinct entries of each vertex's list -> histogram (block-aggregated in shared memory)
__global__ void valence_hist_kernel(const int32_t* off, const int32_t* cnt, const int32_t* nbr, int64_t nv,
                                    unsigned* hist) {
  __shared__ unsigned h[kValenceBins];
  for (int b = threadIdx.x; b < kValenceBins; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* L = nbr + off[v];
    const int n = cnt[v];
    int distinct = 0;
    for (int x = 0; x < n; x++) {
      bool seen = false;
      for (int y = 0; y < x && !seen; y++) seen = L[y] == L[x];
      distinct += !seen;
    }
    atomicAdd(h + (distinct < kValenceBins ? distinct : kValenceBins - 1), 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kValenceBins; b += blockDim.x)
    if (h[b]) atomicAdd(hist + b, h[b]);
}

// device copies of a mesh's positions and faces (a host mesh is copied in; a device mesh is used
// in place)
struct DevMesh {
  const float* v = nullptr;
  const int32_t* faces = nullptr;
  std::vector<void*> owned;
  ~DevMesh() {
    for (void* p : owned) cudaFree(p);
  }
};

tmc_status dev_mesh(tmc_ctx* ctx, const tmc_mesh* m, int P, DevMesh& d) {
  const int32_t* faces = P == 4 ? m->quads : m->tris;
  const int64_t nf = P == 4 ? m->nr_q : m->nr_t;
  (void)nf;
  if (!faces && m->nr_v > 0) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, P == 4 ? "the mesh has no quads" : "the mesh has no triangles");
  if (m->on_device) {
    d.v = m->v;
    d.faces = faces;
    return TMC_OK;
  }
  void* pv = nullptr;
  void* pf = nullptr;
  cudaError_t e = cudaMalloc(&pv, std::max<int64_t>(3 * m->nr_v, 1) * sizeof(float));
  if (e == cudaSuccess) d.owned.push_back(pv);
  if (e == cudaSuccess) e = cudaMalloc(&pf, std::max<int64_t>(P * nf, 1) * sizeof(int32_t));
  if (e == cudaSuccess) d.owned.push_back(pf);
  cudaStream_t st = ctx_stream(ctx);
  if (e == cudaSuccess && m->nr_v) e = cudaMemcpyAsync(pv, m->v, 3 * m->nr_v * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nf) e = cudaMemcpyAsync(pf, faces, P * nf * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  d.v = (const float*)pv;
  d.faces = (const int32_t*)pf;
  return TMC_OK;
}

unsigned grid_of(int64_t n, int sms) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 8));
}

}  // namespace
}  // namespace tmc

using namespace tmc;

extern "C" {

tmc_status tmc_mesh_quality(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, float* quality, double summary[3]) {
  if (!ctx || !mesh) return TMC_ERR_INVALID_ARG;
  if (faces != TMC_FACES_QUADS && faces != TMC_FACES_TRIS) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "unknown face kind");
  const int P = faces == TMC_FACES_QUADS ? 4 : 3;
  const int64_t nf = P == 4 ? mesh->nr_q : mesh->nr_t;
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  DevMesh d;
  tmc_status s = dev_mesh(ctx, mesh, P, d);
  if (s) return s;
  cudaStream_t st = ctx_stream(ctx);
  float* q = nullptr;
  unsigned* red = nullptr;  // [0] min bits, [1] max bits, then a double sum at [2..3]
  e = cudaMalloc(&q, std::max<int64_t>(nf, 1) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&red, 4 * sizeof(unsigned));
  const unsigned init[4] = {0x7f800000u /* +inf */, 0u, 0u, 0u};
  if (e == cudaSuccess) e = cudaMemcpyAsync(red, init, sizeof init, cudaMemcpyHostToDevice, st);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx_device(ctx));
  if (e == cudaSuccess && nf > 0) {
    quality_kernel<<<grid_of(nf, sms), 256, 0, st>>>(d.v, d.faces, P, nf, q, red, red + 1, (double*)(red + 2));
    e = cudaGetLastError();
    ctx_count_launches(ctx, 1);
  }
  unsigned h_red[4] = {0, 0, 0, 0};
  if (e == cudaSuccess && quality && nf > 0) e = cudaMemcpyAsync(quality, q, nf * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_red, red, sizeof h_red, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (q) cudaFree(q);
  if (red) cudaFree(red);
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  if (summary) {
    float mn, mx;
    double sum;
    std::memcpy(&mn, &h_red[0], 4);
    std::memcpy(&mx, &h_red[1], 4);
    std::memcpy(&sum, &h_red[2], 8);
    summary[0] = nf > 0 ? mn : 0.0;
    summary[1] = nf > 0 ? mx : 0.0;
    summary[2] = nf > 0 ? sum / (double)nf : 0.0;
  }
  return TMC_OK;
}

tmc_status tmc_mesh_valence(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, uint32_t hist[100], int32_t* len) {
  if (!ctx || !mesh || !hist) return TMC_ERR_INVALID_ARG;
  if (faces != TMC_FACES_QUADS && faces != TMC_FACES_TRIS) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "unknown face kind");
  const int P = faces == TMC_FACES_QUADS ? 4 : 3;
  const int64_t nf = P == 4 ? mesh->nr_q : mesh->nr_t;
  const int64_t nv = mesh->nr_v;
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  DevMesh d;
  tmc_status s = dev_mesh(ctx, mesh, P, d);
  if (s) return s;
  cudaStream_t st = ctx_stream(ctx);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx_device(ctx));
  const int64_t nvb = std::max<int64_t>(nv, 1);
  int32_t *cnt = nullptr, *off = nullptr, *cursor = nullptr, *nbr = nullptr;
  unsigned long long *tiles = nullptr, *total = nullptr;
  unsigned* dh = nullptr;
  e = cudaMalloc(&cnt, nvb * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&off, nvb * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&cursor, nvb * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&nbr, std::max<int64_t>(2 * P * nf, 1) * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&tiles, (scan_tiles(nvb) + 2) * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&total, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&dh, kValenceBins * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, nvb * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, nvb * sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dh, 0, kValenceBins * sizeof(unsigned), st);
  if (e == cudaSuccess && nv > 0) {
    int k = 0;
    if (nf > 0) {
      nbr_count_kernel<<<grid_of(P * nf, sms), 256, 0, st>>>(d.faces, P, nf, cnt);
      k += 1 + scan_i32(cnt, nv, off, tiles, total, st);
      nbr_scatter_kernel<<<grid_of(P * nf, sms), 256, 0, st>>>(d.faces, P, nf, off, cursor, nbr);
      k++;
    } else {
      e = cudaMemsetAsync(off, 0, nvb * sizeof(int32_t), st);
    }
    valence_hist_kernel<<<grid_of(nv, sms), 256, 0, st>>>(off, cnt, nbr, nv, dh);
    ctx_count_launches(ctx, k + 1);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  unsigned h_hist[kValenceBins];
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_hist, dh, sizeof h_hist, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (void* p : {(void*)cnt, (void*)off, (void*)cursor, (void*)nbr, (void*)tiles, (void*)total, (void*)dh})
    if (p) cudaFree(p);
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  int last = 0;
  for (int b = 0; b < kValenceBins; b++) {
    hist[b] = h_hist[b];
    if (h_hist[b] > 0) last = b;
  }
  if (len) *len = nv > 0 ? last + 1 : 0;
  return TMC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// Mesh check: the counts tmc::MarchingCubes::connectivity (mc/MarchingCubes.cpp:1769-2226) reports,
// computed in parallel.  The reference walks the triangles depth-first from each unvisited one,
// counts the components it starts and flips every triangle whose orientation disagrees with its
// visited neighbour; here the components come from a union-find over the halfedge twins and the
// orientation is checked edge by edge (a twin pair that runs its edge in the same direction is a
// defect).  On a consistently oriented mesh both report no correction; the component counts agree
// whenever each edge has at most two faces (the reference links a face only to the first other
// face it finds on an edge).
// ------------------------------------------------------------------------------------------------
namespace tmc {
namespace {

constexpr int kFindSteps = 1 << 20;  // bound on one find / link loop (never reached: see below)

// root of x with path halving; gives up (returns -1) after kFindSteps steps
__device__ __forceinline__ int32_t uf_find(int32_t* parent, int32_t x) {
  for (int s = 0; s < kFindSteps; s++) {
    const int32_t p = parent[x];
    if (p == x) return x;
    const int32_t gp = parent[p];
    if (gp != p) atomicCAS(parent + x, p, gp);  // halve the path; losing the race is harmless
    x = gp;
  }
  return -1;
}

// Union by linking the larger root under the smaller one (a root's parent only ever decreases, so
// every loop makes progress); each step is bounded all the same.
__device__ __forceinline__ bool uf_union(int32_t* parent, int32_t a, int32_t b) {
  for (int s = 0; s < kFindSteps; s++) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a < 0 || b < 0) return false;
    if (a == b) return true;
    if (a < b) {
      const int32_t t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(parent + a, a, b) == a) return true;
  }
  return false;
}

// counts[0] orientation defects, [1] boundary edges, [2] non-manifold halfedges, [3] degenerate
// faces, [4] gave-up unions
__global__ void check_edges_kernel(const int32_t* faces, int P, int64_t nf, const int32_t* twin, const uint8_t* flag,
                                   int32_t* parent, uint8_t* vbound, unsigned long long* counts) {
  const int64_t nh = nf * P;
  unsigned long long c[5] = {0, 0, 0, 0, 0};
  for (int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = h / P;
    const int r = (int)(h - f * P);
    const int a = faces[h], b = faces[f * P + (r + 1) % P];
    if (r == 0) {
      bool deg = false;
      for (int x = 0; x < P; x++)
        for (int y = x + 1; y < P; y++) deg = deg || faces[f * P + x] == faces[f * P + y];
      c[3] += deg;
    }
    if (flag[h]) c[2]++;
    const int32_t t = twin[h];
    if (t < 0) {
      c[1]++;
      vbound[a] = 1;
      vbound[b] = 1;
      continue;
    }
    if (t < h) continue;  // each pair once
    if (faces[t] == a) c[0]++;  // the twin starts where h starts: both faces run the edge one way
    if (!uf_union(parent, (int32_t)f, (int32_t)(t / P))) c[4]++;
  }
  for (int q = 0; q < 5; q++) {
    unsigned long long x = c[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(counts + q, x);
  }
}

__global__ void iota_kernel(int32_t* p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = (int32_t)i;
}
// counts[5] components (roots), counts[6] boundary vertices
__global__ void count_roots_kernel(const int32_t* parent, int64_t nf, const uint8_t* vbound, int64_t nv,
                                   unsigned long long* counts) {
  unsigned long long roots = 0, bv = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf || i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < nf) roots += parent[i] == (int32_t)i;
    if (i < nv) bv += vbound[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    roots += __shfl_down_sync(0xffffffffu, roots, o);
    bv += __shfl_down_sync(0xffffffffu, bv, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (roots) atomicAdd(counts + 5, roots);
    if (bv) atomicAdd(counts + 6, bv);
  }
}

}  // namespace
}  // namespace tmc

extern "C" tmc_status tmc_mesh_check(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, int64_t report[6]) {
  if (!ctx || !mesh || !report) return TMC_ERR_INVALID_ARG;
  if (faces != TMC_FACES_QUADS && faces != TMC_FACES_TRIS) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "unknown face kind");
  const int P = faces == TMC_FACES_QUADS ? 4 : 3;
  const int64_t nf = P == 4 ? mesh->nr_q : mesh->nr_t;
  const int64_t nv = mesh->nr_v;
  if (4 * nf >= (int64_t)0x7fffffff) return ctx_fail(ctx, TMC_ERR_CAPACITY, "too many faces for 32-bit halfedge ids");
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  DevMesh d;
  tmc_status s = dev_mesh(ctx, mesh, P, d);
  if (s) return s;
  for (int q = 0; q < 6; q++) report[q] = 0;
  if (nf == 0 || nv == 0) return TMC_OK;
  cudaStream_t st = ctx_stream(ctx);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx_device(ctx));
  const int64_t nh = nf * P;
  std::vector<void*> bufs;
  auto get = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) bufs.push_back(p);
    return p;
  };
  HeOut ho{(int32_t*)get(nh * 4), (uint8_t*)get(nh), (int32_t*)get(nv * 4)};
  HeWork w{(int32_t*)get(nv * 4), (int32_t*)get(nv * 4), (int32_t*)get(nh * 4), (int2*)get(nh * 8),
           (unsigned long long*)get(nv * 8), (unsigned long long*)get((scan_tiles(nv) + 2) * 8),
           (unsigned long long*)get(16), (unsigned long long*)get(16)};
  int32_t* parent = (int32_t*)get(nf * 4);
  uint8_t* vbound = (uint8_t*)get(nv);
  unsigned long long* counts = (unsigned long long*)get(8 * 8);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.non_manifold, 0, 16, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(vbound, 0, nv, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, 64, st);
  unsigned long long h_counts[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (e == cudaSuccess) {
    int k = build_halfedges(d.faces, P, nf, nv, ho, w, sms, st, false);  // twins and flags only
    iota_kernel<<<grid_of(nf, sms), 256, 0, st>>>(parent, nf);
    check_edges_kernel<<<grid_of(nh, sms), 256, 0, st>>>(d.faces, P, nf, ho.twin, ho.flag, parent, vbound, counts);
    count_roots_kernel<<<grid_of(std::max(nf, nv), sms), 256, 0, st>>>(parent, nf, vbound, nv, counts);
    ctx_count_launches(ctx, k + 3);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_counts, counts, sizeof h_counts, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (void* p : bufs) cudaFree(p);
  if (e != cudaSuccess) return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  if (h_counts[4]) return ctx_fail(ctx, TMC_ERR_TIMEOUT, "a union-find step gave up after its bound");
  report[0] = (int64_t)h_counts[5];  // components
  report[1] = (int64_t)h_counts[0];  // orientation defects
  report[2] = (int64_t)h_counts[1];  // boundary edges
  report[3] = (int64_t)h_counts[2];  // non-manifold halfedges
  report[4] = (int64_t)h_counts[3];  // degenerate faces
  report[5] = (int64_t)h_counts[6];  // boundary vertices
  return TMC_OK;
}
