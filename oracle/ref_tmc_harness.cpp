// Test-infrastructure harness around the reference's own CPU topologically correct Marching
// Cubes (mc/MarchingCubes.cpp), compiled from the reference sources in place by
// oracle/Makefile into oracle/_ref/.  Only tests and the fixture generator load it.
//
// The harness reproduces what MarchingCubes::operator() does after reading a volume
// (mc/MarchingCubes.cpp:12-78): UGrid::init with the bounding box, scalars as doubles,
// UGrid::gradient() (one-sided differences at the border, :1451), then t_mc(i0) (:151).
// The input here is an in-memory float32 field instead of a ushort file.
#include <algorithm>
#include <cstdlib>
#include <string>
#include <array>
#include <bitset>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <map>
#include <sstream>
#include <vector>

#define private public
#include "MarchingCubes.h"
#undef private

namespace {
struct QuietStdout {
  std::streambuf* old;
  std::streambuf* old_err;
  std::ostringstream sink;
  QuietStdout() { old = std::cout.rdbuf(sink.rdbuf()); old_err = std::cerr.rdbuf(sink.rdbuf()); }
  ~QuietStdout() { std::cout.rdbuf(old); std::cerr.rdbuf(old_err); }
};
struct TmcResult {
  std::vector<double> v, n;
  std::vector<int> tris;
};
}  // namespace

extern "C" {

void* ref_tmc_run(int nx, int ny, int nz, const double* origin, const double* spacing,
                  const float* field, double iso) {
  QuietStdout q;
  auto* mc = new tmc::MarchingCubes();
  std::array<tmc::MarchingCubes::Point, 8> bb;
  const double xs[2] = {origin[0], origin[0] + spacing[0] * (nx - 1.)};
  const double ys[2] = {origin[1], origin[1] + spacing[1] * (ny - 1.)};
  const double zs[2] = {origin[2], origin[2] + spacing[2] * (nz - 1.)};
  for (int c = 0; c < 8; c++) bb[c] = tmc::MarchingCubes::Point{{xs[c & 1], ys[(c >> 1) & 1], zs[(c >> 2) & 1]}};
  mc->m_nx = nx;
  mc->m_ny = ny;
  mc->m_nz = nz;
  mc->m_dx = spacing[0];
  mc->m_dy = spacing[1];
  mc->m_dz = spacing[2];
  mc->m_ugrid.init(nx, ny, nz, bb);
  mc->m_ugrid.set_dx(spacing[0]);
  mc->m_ugrid.set_dy(spacing[1]);
  mc->m_ugrid.set_dz(spacing[2]);
  const size_t n = (size_t)nx * ny * nz;
  for (size_t s = 0; s < n; s++) mc->m_ugrid.scalar((int)s, (double)field[s]);
  mc->m_ugrid.gradient();
  mc->t_mc(iso);
  auto* r = new TmcResult();
  for (auto& p : mc->m_points) { r->v.push_back(p[0]); r->v.push_back(p[1]); r->v.push_back(p[2]); }
  for (auto& p : mc->m_pnorms) { r->n.push_back(p[0]); r->n.push_back(p[1]); r->n.push_back(p[2]); }
  for (auto& t : mc->m_triangles) { r->tris.push_back(t.v[0]); r->tris.push_back(t.v[1]); r->tris.push_back(t.v[2]); }
  delete mc;
  return r;
}

void ref_tmc_sizes(void* h, int64_t* out2) {
  auto* r = (TmcResult*)h;
  out2[0] = (int64_t)r->v.size() / 3;
  out2[1] = (int64_t)r->tris.size() / 3;
}

void ref_tmc_copy(void* h, double* v, double* n, int* tris) {
  auto* r = (TmcResult*)h;
  if (v) std::memcpy(v, r->v.data(), r->v.size() * sizeof(double));
  if (n) std::memcpy(n, r->n.data(), r->n.size() * sizeof(double));
  if (tris) std::memcpy(tris, r->tris.data(), r->tris.size() * sizeof(int));
}

void ref_tmc_free(void* h) { delete (TmcResult*)h; }

// The reference's connectivity() (mc/MarchingCubes.cpp:1769-2226) on the t_mc mesh of a field: it
// reports the components it found and the orientations it changed on stdout; out2 gets both.
void ref_tmc_connectivity(int nx, int ny, int nz, const double* origin, const double* spacing, const float* field,
                          double iso, int64_t* out2) {
  out2[0] = out2[1] = -1;
  std::string text;
  // the set-up of ref_tmc_run, keeping the MarchingCubes object for connectivity()
  QuietStdout q;
  tmc::MarchingCubes mc;
  std::array<tmc::MarchingCubes::Point, 8> bb;
  const double xs[2] = {origin[0], origin[0] + spacing[0] * (nx - 1.)};
  const double ys[2] = {origin[1], origin[1] + spacing[1] * (ny - 1.)};
  const double zs[2] = {origin[2], origin[2] + spacing[2] * (nz - 1.)};
  for (int c = 0; c < 8; c++) bb[c] = tmc::MarchingCubes::Point{{xs[c & 1], ys[(c >> 1) & 1], zs[(c >> 2) & 1]}};
  mc.m_nx = nx;
  mc.m_ny = ny;
  mc.m_nz = nz;
  mc.m_dx = spacing[0];
  mc.m_dy = spacing[1];
  mc.m_dz = spacing[2];
  mc.m_ugrid.init(nx, ny, nz, bb);
  mc.m_ugrid.set_dx(spacing[0]);
  mc.m_ugrid.set_dy(spacing[1]);
  mc.m_ugrid.set_dz(spacing[2]);
  const size_t n = (size_t)nx * ny * nz;
  for (size_t s = 0; s < n; s++) mc.m_ugrid.scalar((int)s, (double)field[s]);
  mc.m_ugrid.gradient();
  mc.t_mc(iso);
  mc.connectivity();
  text = q.sink.str();
  const auto grab = [&](const std::string& before, const std::string& after) -> int64_t {
    const size_t b = text.find(before);
    if (b == std::string::npos) return -1;
    const size_t s0 = b + before.size();
    const size_t e = text.find(after, s0);
    if (e == std::string::npos) return -1;
    return std::atoll(text.substr(s0, e - s0).c_str());
  };
  out2[0] = grab(" connectivity found ", " components");
  out2[1] = grab(" connectivity has changed ", " triangle orientations");
}

// The reference's own file path: MarchingCubes::operator() reads a ushort volume file
// (mc/MarchingCubes.cpp:12-78) and writes its OBJ and OFF files (:98-141).
void ref_tmc_files(double iso, const char* volume, const char* obj, const char* off) {
  QuietStdout q;
  tmc::MarchingCubes mc;
  mc(iso, std::string(volume), false, true, std::string(obj), true, std::string(off));
}

}  // extern "C"
