// C++ adapters with the reference's call signatures, implemented on the C ABI (tmc_gb300.h).
// Header-only; link against libtmc_gb300.so.  Existing callers switch by changing the namespace:
//
//   dmc::DualMarchingCubes::dualMC            -> tmc_gb300::dmc::DualMarchingCubes::dualMC
//       (cpp_dmc/DualMarchingCubes.h:163-165: double isovalue, UniformGrid&, appends v/n/tris/quads)
//   p_mc::DualMarchingCubes::dualMC           -> tmc_gb300::p_mc::DualMarchingCubes::dualMC
//       (dmc/DualMarchingCubes.h:74-77: float isovalue, array outputs, config map)
//   p_mc::MarchingCubes::mc_sharedvertex/mc_halfedge -> tmc_gb300::p_mc::MarchingCubes::...
//       (cuda_tmc/MarchingCubes.h:60,71: volume file in, new[] outputs the caller delete[]s)
//
// Errors: the reference exits or prints; the adapters throw tmc_gb300::Error carrying the status.
#pragma once

#include <array>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "tmc_gb300.h"

namespace tmc_gb300 {

struct Error : std::runtime_error {
  tmc_status status;
  Error(tmc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// One context per adapter object (thread-compatible, like the reference objects).
class Context {
 public:
  explicit Context(int device = 0) {
    const tmc_status s = tmc_ctx_create(device, nullptr, &ctx_);
    if (s != TMC_OK) throw Error(s, "tmc_ctx_create failed");
  }
  ~Context() {
    if (ctx_) tmc_ctx_destroy(ctx_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  tmc_ctx* get() const { return ctx_; }
  void check(tmc_status s) const {
    if (s != TMC_OK) throw Error(s, tmc_last_error(ctx_));
  }

 private:
  tmc_ctx* ctx_ = nullptr;
};

// Volume file in the reference's format (mc/MarchingCubes.cpp:22-66, cuda_tmc/MarchingCubes.cu:3363-3407):
// three ushort dimensions, three float spacings, then ushort samples (x fastest).
struct VolumeFile {
  int nx = 0, ny = 0, nz = 0;
  double spacing[3] = {1, 1, 1};
  std::vector<float> data;
  static VolumeFile read_ushort(const std::string& path) {
    VolumeFile v;
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(TMC_ERR_INVALID_ARG, "can't open volume file " + path);
    unsigned short d[3];
    float s[3];
    if (std::fread(d, sizeof(unsigned short), 3, f) != 3 || std::fread(s, sizeof(float), 3, f) != 3) {
      std::fclose(f);
      throw Error(TMC_ERR_INVALID_ARG, "truncated volume header " + path);
    }
    v.nx = d[0];
    v.ny = d[1];
    v.nz = d[2];
    for (int q = 0; q < 3; q++) v.spacing[q] = s[q];
    const size_t n = (size_t)v.nx * v.ny * v.nz;
    std::vector<unsigned short> buf(n);
    if (std::fread(buf.data(), sizeof(unsigned short), n, f) != n) {
      std::fclose(f);
      throw Error(TMC_ERR_INVALID_ARG, "truncated volume data " + path);
    }
    std::fclose(f);
    v.data.assign(buf.begin(), buf.end());
    return v;
  }
  tmc_volume view() const {
    tmc_volume t{};
    t.nx = nx;
    t.ny = ny;
    t.nz = nz;
    t.origin[0] = t.origin[1] = t.origin[2] = 0.0;  // the reference places the file grid at the origin
    for (int q = 0; q < 3; q++) t.spacing[q] = spacing[q];
    t.data = data.data();
    t.on_device = 0;
    return t;
  }
};

namespace detail {
struct MeshGuard {
  tmc_ctx* ctx;
  tmc_mesh m{};
  explicit MeshGuard(tmc_ctx* c) : ctx(c) {}
  ~MeshGuard() { tmc_mesh_free(ctx, &m); }
};
}  // namespace detail

// ------------------------------------------------------------------------------------------------
// cpp_dmc-style CPU interface
// ------------------------------------------------------------------------------------------------
namespace dmc {

struct Vector {
  double p[3]{0, 0, 0};
  double& operator[](size_t i) { return p[i]; }
  const double& operator[](size_t i) const { return p[i]; }
};

// Uniform grid holding float32 samples (the reference holds doubles; every sample it extracts
// from started as a float or ushort, so float32 storage loses nothing).
class UniformGrid {
 public:
  using BBox = std::array<Vector, 8>;
  void init(int nx, int ny, int nz, const BBox& bb) {
    nx_ = nx;
    ny_ = ny;
    nz_ = nz;
    origin_[0] = bb[0][0];
    origin_[1] = bb[0][1];
    origin_[2] = bb[0][2];
    d_[0] = (bb[7][0] - bb[0][0]) / (nx - 1.0);
    d_[1] = (bb[7][1] - bb[0][1]) / (ny - 1.0);
    d_[2] = (bb[7][2] - bb[0][2]) / (nz - 1.0);
    data_.assign((size_t)nx * ny * nz, 0.0f);
  }
  void set_dx(double d) { d_[0] = d; }
  void set_dy(double d) { d_[1] = d; }
  void set_dz(double d) { d_[2] = d; }
  void scalar(int i, int j, int k, double val) { data_[((size_t)k * ny_ + j) * nx_ + i] = (float)val; }
  void scalar(int gindex, double val) { data_[(size_t)gindex] = (float)val; }
  double scalar(int i, int j, int k) const { return data_[((size_t)k * ny_ + j) * nx_ + i]; }
  int x_size() const { return nx_; }
  int y_size() const { return ny_; }
  int z_size() const { return nz_; }
  // normals from the negated estimated gradient, as UniformGrid::init(file) sets them up
  void flip_gradient(bool on = true) { flip_ = on; }
  tmc_volume view() const {
    tmc_volume t{};
    t.nx = nx_;
    t.ny = ny_;
    t.nz = nz_;
    for (int q = 0; q < 3; q++) {
      t.origin[q] = origin_[q];
      t.spacing[q] = d_[q];
    }
    t.data = data_.data();
    t.on_device = 0;
    return t;
  }
  bool flipped() const { return flip_; }

 private:
  int nx_ = 0, ny_ = 0, nz_ = 0;
  double origin_[3]{0, 0, 0}, d_[3]{1, 1, 1};
  bool flip_ = false;
  std::vector<float> data_;
};

class DualMarchingCubes {
 public:
  explicit DualMarchingCubes(int device = 0) : ctx_(device) {}
  // cpp_dmc/DualMarchingCubes.h:163-165.  Outputs are appended, as the reference does; vertex
  // positions and normals are float64 (positions bit-equal to the reference's).
  void dualMC(const double i0, UniformGrid& ugrid, std::vector<Vector>& v, std::vector<Vector>& n,
              std::vector<int>& triangles, std::vector<int>& quads, const bool sFlag) {
    const tmc_volume vol = ugrid.view();
    detail::MeshGuard g(ctx_.get());
    uint32_t flags = TMC_OUT_HOST | TMC_OUT_POS_F64 | TMC_OUT_TRIANGLES | (sFlag ? TMC_DMC_SIMPLIFY : 0u) |
                     (ugrid.flipped() ? TMC_GRAD_FLIP : 0u);
    ctx_.check(tmc_dmc_extract(ctx_.get(), &vol, i0, flags, &g.m));
    const size_t base = v.size();
    v.resize(base + (size_t)g.m.nr_v);
    n.resize(base + (size_t)g.m.nr_v);
    for (int64_t i = 0; i < g.m.nr_v; i++)
      for (int d = 0; d < 3; d++) {
        v[base + i][d] = g.m.v64[3 * i + d];
        n[base + i][d] = g.m.n[3 * i + d];
      }
    quads.insert(quads.end(), g.m.quads, g.m.quads + 4 * g.m.nr_q);
    triangles.insert(triangles.end(), g.m.tris, g.m.tris + 3 * g.m.nr_t);
  }

 private:
  Context ctx_;
};

}  // namespace dmc

// ------------------------------------------------------------------------------------------------
// GPU-reference-style interfaces
// ------------------------------------------------------------------------------------------------
namespace p_mc {

class DualMarchingCubes {
 public:
  explicit DualMarchingCubes(int device = 0) : ctx_(device) {}
  // set the volume (dmc/DualMarchingCubes.h:84-90 init): float samples, x fastest
  void init(int nx, int ny, int nz, const std::vector<float>& data, const double origin[3], const double spacing[3]) {
    vol_ = tmc_volume{};
    vol_.nx = nx;
    vol_.ny = ny;
    vol_.nz = nz;
    for (int q = 0; q < 3; q++) {
      vol_.origin[q] = origin[q];
      vol_.spacing[q] = spacing[q];
    }
    data_ = data;
    vol_.data = data_.data();
  }
  // dmc/DualMarchingCubes.h:74-77.  config keys as the reference: "p3X3YColor", "p3X3YOld",
  // "p3333", "halfedge-datastructure" (non-zero = on).
  void dualMC(float i0, std::vector<std::array<float, 3>>& v, std::vector<std::array<float, 3>>& n,
              std::vector<std::array<int, 3>>& t, std::vector<std::array<int, 4>>& q,
              std::vector<std::array<int, 4>>& he, std::vector<int>& hef, std::vector<int>& hev,
              std::map<std::string, int>& config) {
    auto on = [&](const char* k) { return config.count(k) && config[k] != 0; };
    uint32_t flags = TMC_OUT_HOST | TMC_OUT_TRIANGLES;
    if (on("p3X3YColor")) flags |= TMC_DMC_P3X3Y_COLOR;
    if (on("p3X3YOld")) flags |= TMC_DMC_P3X3Y_ISOLATED;
    if (on("p3333")) flags |= TMC_DMC_P3333;
    if (on("halfedge-datastructure")) flags |= TMC_OUT_HALFEDGES;
    detail::MeshGuard g(ctx_.get());
    ctx_.check(tmc_dmc_extract(ctx_.get(), &vol_, i0, flags, &g.m));
    v.resize((size_t)g.m.nr_v);
    n.resize((size_t)g.m.nr_v);
    for (int64_t i = 0; i < g.m.nr_v; i++)
      for (int d = 0; d < 3; d++) {
        v[i][d] = g.m.v[3 * i + d];
        n[i][d] = g.m.n[3 * i + d];
      }
    q.resize((size_t)g.m.nr_q);
    std::memcpy(q.data(), g.m.quads, sizeof(int) * 4 * g.m.nr_q);
    t.resize((size_t)g.m.nr_t);
    std::memcpy(t.data(), g.m.tris, sizeof(int) * 3 * g.m.nr_t);
    he.resize((size_t)g.m.nr_he);
    if (g.m.nr_he) std::memcpy(he.data(), g.m.he, sizeof(int) * 4 * g.m.nr_he);
    hef.assign(g.m.he_f ? g.m.he_f : nullptr, g.m.he_f ? g.m.he_f + g.m.nr_q : nullptr);
    hev.assign(g.m.he_v ? g.m.he_v : nullptr, g.m.he_v ? g.m.he_v + g.m.nr_v : nullptr);
  }

 private:
  Context ctx_;
  tmc_volume vol_{};
  std::vector<float> data_;
};

class MarchingCubes {
 public:
  explicit MarchingCubes(int device = 0) : ctx_(device) {}
  // cuda_tmc/MarchingCubes.h:60: outputs allocated with new[], freed by the caller with delete[]
  void mc_sharedvertex(float i0, const std::string& file, int& nr_v, float** vertices, float** normals, int& nr_t,
                       int** triangles) {
    const VolumeFile vf = VolumeFile::read_ushort(file);
    const tmc_volume vol = vf.view();
    detail::MeshGuard g(ctx_.get());
    ctx_.check(tmc_tmc_sharedvertex(ctx_.get(), &vol, i0, TMC_OUT_HOST, &g.m));
    nr_v = (int)g.m.nr_v;
    nr_t = (int)g.m.nr_t;
    *vertices = copy_new(g.m.v, 3 * g.m.nr_v);
    *normals = copy_new(g.m.n, 3 * g.m.nr_v);
    *triangles = copy_new(g.m.tris, 3 * g.m.nr_t);
  }
  // cuda_tmc/MarchingCubes.h:71: halfedges as int4-like records {origin, face, next, twin}
  void mc_halfedge(float i0, const std::string& file, int& nr_v, float** vertices, float** normals, int& nr_t,
                   int** he, int** hev, int** hef) {
    const VolumeFile vf = VolumeFile::read_ushort(file);
    const tmc_volume vol = vf.view();
    detail::MeshGuard g(ctx_.get());
    ctx_.check(tmc_tmc_halfedge(ctx_.get(), &vol, i0, TMC_OUT_HOST, &g.m));
    nr_v = (int)g.m.nr_v;
    nr_t = (int)g.m.nr_t;
    *vertices = copy_new(g.m.v, 3 * g.m.nr_v);
    *normals = copy_new(g.m.n, 3 * g.m.nr_v);
    *he = copy_new(g.m.he, 4 * g.m.nr_he);
    *hev = copy_new(g.m.he_v, g.m.nr_v);
    *hef = copy_new(g.m.he_f, g.m.nr_t);
  }

 private:
  template <typename T>
  static T* copy_new(const T* src, int64_t count) {
    T* p = new T[count > 0 ? count : 1];
    if (count > 0) std::memcpy(p, src, sizeof(T) * (size_t)count);
    return p;
  }
  Context ctx_;
};

}  // namespace p_mc
}  // namespace tmc_gb300
