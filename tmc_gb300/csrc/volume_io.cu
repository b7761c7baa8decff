// Volume files in the reference's formats (loaded into device memory) and OBJ / OFF output of
// meshes in the reference's text layouts.
//
// Formats (origin 0 in all of them; spacing widened to float64 as the readers do):
//   TMC_FILE_DMC      int32 nx, ny, nz; float64 dx, dy, dz; float32 data
//                     (dmc::UniformGrid::init, cpp_dmc/UniformGrid.cpp:3-45)
//   TMC_FILE_INT_F32  int32 nx, ny, nz; float32 dx, dy, dz; float32 data
//                     (readFromFile<float>, cpp_dmc/Volumes.h:47-105; readDataFromFile<float>,
//                     dmc/UniformGrid.h:431-468)
//   TMC_FILE_INT_U16  the same header with uint16 data (the <ushort> instances: CT / MRI scans)
//   TMC_FILE_U16      uint16 nx, ny, nz; float32 dx, dy, dz; uint16 data
//                     (MarchingCubes::operator(), mc/MarchingCubes.cpp:22-66;
//                     p_mc::MarchingCubes::readDataFromFile, cuda_tmc/MarchingCubes.cu:3363-3407)
// The data is x fastest, as the extraction entry points expect.  uint16 data is copied to the
// device as it is (2 bytes per voxel over PCIe / C2C) and widened to float32 there by a
// conversion kernel; every uint16 value is exact in float32.  The reference readers convert on the
// host (and exit the process on a bad file); these return a status.
//
// Writers:
//   TMC_OBJ_DMC_TRIS / TMC_OBJ_DMC_QUADS  cpp_dmc/main.cpp:33-87: "v"/"vn" lines with the stream's
//       default formatting (printf %g), faces "f a//a ..." (1-based)
//   TMC_OBJ_TMC  mc/MarchingCubes.cpp:98-118: "v"/"vn" with 7 fixed decimals, triangle faces
//       "f a//a b//b c//b" -- the reference writes the second vertex's index as the third normal
//       index; kept so that files compare equal to the reference's
//   OFF  mc/MarchingCubes.cpp:123-141: "OFF", counts, points (%g), faces "3 a b c" (0-based);
//       a quad mesh writes "4 a b c d"
// Positions come from the float64 array when the mesh has one, else from the float32 one.
#include <algorithm>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/tmc_gb300.h"
#include "common.cuh"
#include "ctx_access.h"
#include "generators.cuh"

namespace tmc {
namespace {

// eight uint16 values per thread: one 16-byte load, two 16-byte stores
__global__ void u16_to_f32_kernel(const uint16_t* in, float* out, int64_t n) {
  const int64_t n8 = n / 8;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n8; q += (int64_t)gridDim.x * blockDim.x) {
    const uint4 w = reinterpret_cast<const uint4*>(in)[q];
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
    float4 a, b;
    a.x = (float)(x[0] & 0xFFFFu); a.y = (float)(x[0] >> 16);
    a.z = (float)(x[1] & 0xFFFFu); a.w = (float)(x[1] >> 16);
    b.x = (float)(x[2] & 0xFFFFu); b.y = (float)(x[2] >> 16);
    b.z = (float)(x[3] & 0xFFFFu); b.w = (float)(x[3] >> 16);
    reinterpret_cast<float4*>(out)[2 * q] = a;
    reinterpret_cast<float4*>(out)[2 * q + 1] = b;
  }
  // the last n % 8 values
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n - 8 * n8) out[8 * n8 + t] = (float)in[8 * n8 + t];
}

struct FileInfo {
  int32_t dims[3];
  double spacing[3];
  int64_t offset;  // first data byte
  int elem;        // bytes per value
};

tmc_status read_info(const char* path, int32_t format, FileInfo& fi, char* msg, size_t msg_len) {
  std::FILE* f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) {
    std::snprintf(msg, msg_len, "cannot open volume file %s", path ? path : "(null)");
    return TMC_ERR_INVALID_ARG;
  }
  bool ok = true;
  if (format == TMC_FILE_U16) {
    uint16_t d[3];
    float s[3];
    ok = std::fread(d, 2, 3, f) == 3 && std::fread(s, 4, 3, f) == 3;
    for (int a = 0; a < 3; a++) {
      fi.dims[a] = d[a];
      fi.spacing[a] = (double)s[a];
    }
    fi.offset = 18;
    fi.elem = 2;
  } else if (format == TMC_FILE_DMC || format == TMC_FILE_INT_F32 || format == TMC_FILE_INT_U16) {
    int32_t d[3];
    ok = std::fread(d, 4, 3, f) == 3;
    if (format == TMC_FILE_DMC) {
      double s[3];
      ok = ok && std::fread(s, 8, 3, f) == 3;
      for (int a = 0; a < 3; a++) fi.spacing[a] = s[a];
      fi.offset = 36;
    } else {
      float s[3];
      ok = ok && std::fread(s, 4, 3, f) == 3;
      for (int a = 0; a < 3; a++) fi.spacing[a] = (double)s[a];
      fi.offset = 24;
    }
    for (int a = 0; a < 3; a++) fi.dims[a] = d[a];
    fi.elem = format == TMC_FILE_INT_U16 ? 2 : 4;
  } else {
    std::fclose(f);
    std::snprintf(msg, msg_len, "unknown volume file format %d", format);
    return TMC_ERR_INVALID_ARG;
  }
  int64_t size = -1;
  if (ok && std::fseek(f, 0, SEEK_END) == 0) size = (int64_t)std::ftell(f);
  std::fclose(f);
  if (!ok) {
    std::snprintf(msg, msg_len, "%s: truncated header", path);
    return TMC_ERR_INVALID_ARG;
  }
  for (int a = 0; a < 3; a++) {
    if (fi.dims[a] < 2) {
      std::snprintf(msg, msg_len, "%s: dimension %d is %d (at least 2 points per axis)", path, a, fi.dims[a]);
      return TMC_ERR_INVALID_ARG;
    }
    if (!(fi.spacing[a] > 0) || !std::isfinite(fi.spacing[a])) {
      std::snprintf(msg, msg_len, "%s: spacing %d is not a positive number", path, a);
      return TMC_ERR_INVALID_ARG;
    }
  }
  const int64_t need = fi.offset + (int64_t)fi.dims[0] * fi.dims[1] * fi.dims[2] * fi.elem;
  if (size < need) {
    std::snprintf(msg, msg_len, "%s: %" PRId64 " bytes, the header announces %" PRId64, path, size, need);
    return TMC_ERR_INVALID_ARG;
  }
  return TMC_OK;
}

tmc_status fail_msg(tmc_ctx* ctx, tmc_status s, const char* msg) { return ctx ? ctx_fail(ctx, s, msg) : s; }

// host copy of a mesh's arrays (device meshes are copied back; host meshes are used in place)
struct HostMesh {
  std::vector<float> v, n;
  std::vector<double> v64;
  std::vector<int32_t> q, t;
  const float* pv = nullptr;
  const float* pn = nullptr;
  const double* pv64 = nullptr;
  const int32_t* pq = nullptr;
  const int32_t* pt = nullptr;
};

template <typename T>
cudaError_t fetch(const T* src, size_t count, std::vector<T>& buf, const T*& out) {
  if (!src || count == 0) {
    out = nullptr;
    return cudaSuccess;
  }
  buf.resize(count);
  out = buf.data();
  return cudaMemcpy(buf.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost);
}

tmc_status host_mesh(tmc_ctx* ctx, const tmc_mesh* m, HostMesh& h) {
  if (!m->on_device) {
    h.pv = m->v;
    h.pn = m->n;
    h.pv64 = m->v64;
    h.pq = m->quads;
    h.pt = m->tris;
    return TMC_OK;
  }
  if (!ctx) return TMC_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx_stream(ctx));
  if (e == cudaSuccess) e = fetch(m->v, 3 * (size_t)m->nr_v, h.v, h.pv);
  if (e == cudaSuccess) e = fetch(m->n, 3 * (size_t)m->nr_v, h.n, h.pn);
  if (e == cudaSuccess) e = fetch(m->v64, 3 * (size_t)m->nr_v, h.v64, h.pv64);
  if (e == cudaSuccess) e = fetch(m->quads, 4 * (size_t)m->nr_q, h.q, h.pq);
  if (e == cudaSuccess) e = fetch(m->tris, 3 * (size_t)m->nr_t, h.t, h.pt);
  if (e != cudaSuccess) return fail_msg(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  return TMC_OK;
}

inline double pos(const HostMesh& h, int64_t i) { return h.pv64 ? h.pv64[i] : (double)h.pv[i]; }

}  // namespace
}  // namespace tmc

using namespace tmc;

extern "C" {

tmc_status tmc_volume_file_info(const char* path, int32_t format, int32_t dims[3], double spacing[3],
                                int64_t* data_offset) {
  FileInfo fi;
  char msg[512];
  const tmc_status s = read_info(path, format, fi, msg, sizeof msg);
  if (s) return s;
  for (int a = 0; a < 3; a++) {
    if (dims) dims[a] = fi.dims[a];
    if (spacing) spacing[a] = fi.spacing[a];
  }
  if (data_offset) *data_offset = fi.offset;
  return TMC_OK;
}

tmc_status tmc_field_load(tmc_ctx* ctx, const char* path, int32_t format, tmc_field* out) {
  if (!ctx || !out) return TMC_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  FileInfo fi;
  char msg[512];
  tmc_status s = read_info(path, format, fi, msg, sizeof msg);
  if (s) return ctx_fail(ctx, s, msg);
  const int64_t n = (int64_t)fi.dims[0] * fi.dims[1] * fi.dims[2];
  std::vector<uint8_t> raw((size_t)(n * fi.elem));
  std::FILE* f = std::fopen(path, "rb");
  bool ok = f && std::fseek(f, (long)fi.offset, SEEK_SET) == 0 && std::fread(raw.data(), 1, raw.size(), f) == raw.size();
  if (f) std::fclose(f);
  if (!ok) {
    std::snprintf(msg, sizeof msg, "%s: reading the data failed", path);
    return ctx_fail(ctx, TMC_ERR_INVALID_ARG, msg);
  }
  cudaStream_t st = ctx_stream(ctx);
  float* field = nullptr;
  void* staging = nullptr;
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e == cudaSuccess) e = cudaMalloc(&field, (size_t)n * sizeof(float));
  if (e == cudaSuccess && fi.elem == 4) {
    e = cudaMemcpyAsync(field, raw.data(), raw.size(), cudaMemcpyHostToDevice, st);
  } else if (e == cudaSuccess) {
    e = cudaMalloc(&staging, raw.size());
    if (e == cudaSuccess) e = cudaMemcpyAsync(staging, raw.data(), raw.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx_device(ctx));
      const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(n / 8 + 1, 256), (int64_t)sms * 8));
      u16_to_f32_kernel<<<(unsigned)blocks, 256, 0, st>>>((const uint16_t*)staging, field, n);
      e = cudaGetLastError();
      ctx_count_launches(ctx, 1);
    }
  }
  // the host buffer and the staging buffer are released once the copies are done
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (staging) cudaFree(staging);
  if (e != cudaSuccess) {
    if (field) cudaFree(field);
    return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  }
  out->vol.nx = fi.dims[0];
  out->vol.ny = fi.dims[1];
  out->vol.nz = fi.dims[2];
  for (int a = 0; a < 3; a++) {
    out->vol.origin[a] = 0.0;
    out->vol.spacing[a] = fi.spacing[a];
  }
  out->vol.data = field;
  out->vol.on_device = 1;
  out->priv = field;
  return TMC_OK;
}

tmc_status tmc_field_free(tmc_ctx* ctx, tmc_field* fld) {
  if (!fld) return TMC_ERR_INVALID_ARG;
  if (fld->priv) {
    if (ctx) cudaSetDevice(ctx_device(ctx));
    cudaFree(fld->priv);
  }
  std::memset(fld, 0, sizeof(*fld));
  return TMC_OK;
}

tmc_status tmc_mesh_write_obj(tmc_ctx* ctx, const tmc_mesh* mesh, const char* path, int32_t style) {
  if (!mesh || !path) return fail_msg(ctx, TMC_ERR_INVALID_ARG, "null mesh or path");
  if (style != TMC_OBJ_DMC_TRIS && style != TMC_OBJ_DMC_QUADS && style != TMC_OBJ_TMC)
    return fail_msg(ctx, TMC_ERR_INVALID_ARG, "unknown OBJ style");
  const bool quads = style == TMC_OBJ_DMC_QUADS;
  // the face array the style writes must exist (an empty mesh has none and writes no faces)
  if (mesh->nr_v > 0 && (quads ? !mesh->quads : !mesh->tris))
    return fail_msg(ctx, TMC_ERR_INVALID_ARG, quads ? "the mesh has no quads" : "the mesh has no triangles");
  HostMesh h;
  tmc_status s = host_mesh(ctx, mesh, h);
  if (s) return s;
  std::FILE* f = std::fopen(path, "w");
  if (!f) return fail_msg(ctx, TMC_ERR_INVALID_ARG, "cannot open the output file");
  const int64_t nv = mesh->nr_v;
  if (style == TMC_OBJ_TMC) {
    std::fputs("# Topologically correct and manifold isosurface\n", f);
    for (int64_t i = 0; i < nv; i++)
      std::fprintf(f, "v %.7f %.7f %.7f\n", pos(h, 3 * i), pos(h, 3 * i + 1), pos(h, 3 * i + 2));
    for (int64_t i = 0; i < nv; i++)
      std::fprintf(f, "vn %.7f %.7f %.7f\n", (double)h.pn[3 * i], (double)h.pn[3 * i + 1], (double)h.pn[3 * i + 2]);
    for (int64_t t = 0; t < mesh->nr_t; t++) {
      const int32_t* c = h.pt + 3 * t;
      std::fprintf(f, "f %d//%d %d//%d %d//%d\n", c[0] + 1, c[0] + 1, c[1] + 1, c[1] + 1, c[2] + 1, c[1] + 1);
    }
  } else {
    std::fputs(quads ? "#Dual Marching Cubes, quad only mesh\n" : "#Dual Marching Cubes, triangle mesh\n", f);
    for (int64_t i = 0; i < nv; i++)
      std::fprintf(f, "v %g %g %g\n", pos(h, 3 * i), pos(h, 3 * i + 1), pos(h, 3 * i + 2));
    for (int64_t i = 0; i < nv; i++)
      std::fprintf(f, "vn %g %g %g\n", (double)h.pn[3 * i], (double)h.pn[3 * i + 1], (double)h.pn[3 * i + 2]);
    if (quads) {
      for (int64_t q = 0; q < mesh->nr_q; q++) {
        const int32_t* c = h.pq + 4 * q;
        std::fprintf(f, "f %d//%d %d//%d %d//%d %d//%d\n", c[0] + 1, c[0] + 1, c[1] + 1, c[1] + 1, c[2] + 1,
                     c[2] + 1, c[3] + 1, c[3] + 1);
      }
    } else {
      for (int64_t t = 0; t < mesh->nr_t; t++) {
        const int32_t* c = h.pt + 3 * t;
        std::fprintf(f, "f %d//%d %d//%d %d//%d\n", c[0] + 1, c[0] + 1, c[1] + 1, c[1] + 1, c[2] + 1, c[2] + 1);
      }
    }
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? TMC_OK : fail_msg(ctx, TMC_ERR_INVALID_ARG, "writing the output file failed");
}

tmc_status tmc_mesh_write_off(tmc_ctx* ctx, const tmc_mesh* mesh, const char* path) {
  if (!mesh || !path) return fail_msg(ctx, TMC_ERR_INVALID_ARG, "null mesh or path");
  const bool quads = mesh->nr_t == 0 && mesh->nr_q > 0;
  HostMesh h;
  tmc_status s = host_mesh(ctx, mesh, h);
  if (s) return s;
  std::FILE* f = std::fopen(path, "w");
  if (!f) return fail_msg(ctx, TMC_ERR_INVALID_ARG, "cannot open the output file");
  const int64_t nf = quads ? mesh->nr_q : mesh->nr_t;
  std::fprintf(f, "OFF\n%" PRId64 " %" PRId64 " 0\n", mesh->nr_v, nf);
  for (int64_t i = 0; i < mesh->nr_v; i++)
    std::fprintf(f, "%g %g %g\n", pos(h, 3 * i), pos(h, 3 * i + 1), pos(h, 3 * i + 2));
  for (int64_t q = 0; q < nf; q++) {
    if (quads) {
      const int32_t* c = h.pq + 4 * q;
      std::fprintf(f, "4 %d %d %d %d\n", c[0], c[1], c[2], c[3]);
    } else {
      const int32_t* c = h.pt + 3 * q;
      std::fprintf(f, "3 %d %d %d\n", c[0], c[1], c[2]);
    }
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? TMC_OK : fail_msg(ctx, TMC_ERR_INVALID_ARG, "writing the output file failed");
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// Generated fields: the reference's predefined implicit surfaces (p_mc::UniformGrid::generateVolume
// and its kernel, dmc/UniformGrid.cu:21-217) sampled on [-1, 1]^3 with spacing 2 / (n - 1) in float32.
// The surfaces and their constants are the reference's (they define the test volumes); the
// formulas are written out here per case.
// ------------------------------------------------------------------------------------------------
namespace tmc {
namespace {

__global__ void generate_kernel(GenParams P, int nx, int ny, int nz, float dx, float dy, float dz, float* out) {
  const int64_t n = (int64_t)nx * ny * nz;
  const float d[3] = {dx, dy, dz};
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx), j = (int)((g / nx) % ny), k = (int)(g / ((int64_t)nx * ny));
    out[g] = generated_at(P, d, i, j, k);
  }
}

// The generator's field into new device memory (the stored path of both generation entry points).
tmc_status generate_field(tmc_ctx* ctx, const tmc_generator& gen, tmc_field* out) {
  GenParams P;
  float d[3];
  if (!gen_params(gen, P, d)) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "invalid generator (surface, grid or parameters)");
  const int64_t n = (int64_t)gen.nx * gen.ny * gen.nz;
  float* field = nullptr;
  cudaError_t e = cudaSetDevice(ctx_device(ctx));
  if (e == cudaSuccess) e = cudaMalloc(&field, (size_t)n * sizeof(float));
  if (e == cudaSuccess) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx_device(ctx));
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sms * 16));
    generate_kernel<<<(unsigned)blocks, 256, 0, ctx_stream(ctx)>>>(P, gen.nx, gen.ny, gen.nz, d[0], d[1], d[2], field);
    e = cudaGetLastError();
    ctx_count_launches(ctx, 1);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx_stream(ctx));
  if (e != cudaSuccess) {
    if (field) cudaFree(field);
    return ctx_fail(ctx, TMC_ERR_CUDA, cudaGetErrorString(e));
  }
  out->vol.nx = gen.nx;
  out->vol.ny = gen.ny;
  out->vol.nz = gen.nz;
  for (int a = 0; a < 3; a++) {
    out->vol.origin[a] = -1.0;
    out->vol.spacing[a] = (double)d[a];
  }
  out->vol.data = field;
  out->vol.on_device = 1;
  out->priv = field;
  return TMC_OK;
}

}  // namespace
}  // namespace tmc

extern "C" tmc_status tmc_field_generate(tmc_ctx* ctx, int32_t surface, int32_t nx, int32_t ny, int32_t nz,
                                         tmc_field* out) {
  if (!ctx || !out) return TMC_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  if (surface < TMC_SURF_SPHERE || surface > TMC_SURF_STEINER_ROMAN)
    return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "unknown surface");
  if (nx < 2 || ny < 2 || nz < 2) return ctx_fail(ctx, TMC_ERR_INVALID_ARG, "at least 2 points per axis");
  tmc_generator gen{};
  gen.surface = surface;
  gen.nx = nx;
  gen.ny = ny;
  gen.nz = nz;
  return tmc::generate_field(ctx, gen, out);
}

extern "C" tmc_status tmc_field_generate_ex(tmc_ctx* ctx, const tmc_generator* gen, tmc_field* out) {
  if (!ctx || !out || !gen) return TMC_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  return tmc::generate_field(ctx, *gen, out);
}
