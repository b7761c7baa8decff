// Test-infrastructure harness around the reference's own CPU Dual Marching
// Cubes (cpp_dmc/DualMarchingCubes.cpp, cpp_dmc/UniformGrid.cpp), compiled
// from the reference sources in place by oracle/Makefile into oracle/_ref/.
// Only tests and the fixture generator load the resulting library; it is the
// checker, never the product.
//
// The harness feeds a float32 field (x fastest) into dmc::UniformGrid as
// doubles, estimates the gradient the way the reference does for volumes
// loaded from file (UniformGrid::estimateGradient, cpp_dmc/UniformGrid.cpp:512,
// optionally negated by flip_gradient, :544), runs dualMC
// (cpp_dmc/DualMarchingCubes.cpp:5) and returns flat arrays.  Private stages
// (halfedges, colorFaces, vertexValence) are reached for per-stage checks.
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <list>
#include <map>
#include <sstream>
#include <tuple>
#include <vector>

#define private public
#include "DualMarchingCubes.h"
#undef private

namespace {

struct QuietStdout {
  std::streambuf* old;
  std::streambuf* old_err;
  std::ostringstream sink;
  QuietStdout() { old = std::cout.rdbuf(sink.rdbuf()); old_err = std::cerr.rdbuf(sink.rdbuf()); }
  ~QuietStdout() { std::cout.rdbuf(old); std::cerr.rdbuf(old_err); }
};

struct DmcResult {
  std::vector<double> v, n;
  std::vector<int> tris, quads;
  std::vector<int> he;      // 5 ints per halfedge
  std::vector<int> he_v, he_f;
};

std::vector<DmcResult*> g_results;

void fill_grid(dmc::UniformGrid& ug, int nx, int ny, int nz, const double* origin,
               const double* spacing, const float* field, int flip) {
  dmc::UniformGrid::BBox bb;
  const double x0 = origin[0], y0 = origin[1], z0 = origin[2];
  const double x1 = x0 + spacing[0] * (nx - 1), y1 = y0 + spacing[1] * (ny - 1),
               z1 = z0 + spacing[2] * (nz - 1);
  const double xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
  for (int c = 0; c < 8; c++) bb[c] = dmc::Vector{xs[c & 1], ys[(c >> 1) & 1], zs[(c >> 2) & 1]};
  ug.init(nx, ny, nz, bb);
  // init() derives the spacing from the bounding box; keep the caller's exact value.
  ug.set_dx(spacing[0]);
  ug.set_dy(spacing[1]);
  ug.set_dz(spacing[2]);
  const size_t n = (size_t)nx * ny * nz;
  for (size_t s = 0; s < n; s++) ug.scalar((int)s, (double)field[s]);
  ug.estimateGradient();
  if (flip) ug.flip_gradient();
}

}  // namespace

extern "C" {

// Runs the reference dualMC.  Returns an opaque handle; sizes via ref_dmc_sizes.
void* ref_dmc_run(int nx, int ny, int nz, const double* origin, const double* spacing,
                  const float* field, double iso, int simplify, int flip) {
  QuietStdout q;
  dmc::UniformGrid ug;
  fill_grid(ug, nx, ny, nz, origin, spacing, field, flip);
  dmc::DualMarchingCubes d;
  std::vector<dmc::Vector> v, n;
  auto* r = new DmcResult();
  d.dualMC(iso, ug, v, n, r->tris, r->quads, simplify != 0);
  for (auto& p : v) { r->v.push_back(p[0]); r->v.push_back(p[1]); r->v.push_back(p[2]); }
  for (auto& p : n) { r->n.push_back(p[0]); r->n.push_back(p[1]); r->n.push_back(p[2]); }
  // The final halfedge structure dualMC builds internally (DualMarchingCubes.cpp:77-83)
  std::vector<std::array<int, 5>> he;
  d.halfedges((int)v.size(), r->quads, he, r->he_v, r->he_f);
  for (auto& h : he) for (int k = 0; k < 5; k++) r->he.push_back(h[k]);
  g_results.push_back(r);
  return r;
}

void ref_dmc_sizes(void* h, int64_t* out4) {
  auto* r = (DmcResult*)h;
  out4[0] = (int64_t)r->v.size() / 3;
  out4[1] = (int64_t)r->quads.size() / 4;
  out4[2] = (int64_t)r->tris.size() / 3;
  out4[3] = (int64_t)r->he.size() / 5;
}

void ref_dmc_copy(void* h, double* v, double* n, int* quads, int* tris, int* he, int* he_v, int* he_f) {
  auto* r = (DmcResult*)h;
  if (v) std::memcpy(v, r->v.data(), r->v.size() * sizeof(double));
  if (n) std::memcpy(n, r->n.data(), r->n.size() * sizeof(double));
  if (quads) std::memcpy(quads, r->quads.data(), r->quads.size() * sizeof(int));
  if (tris) std::memcpy(tris, r->tris.data(), r->tris.size() * sizeof(int));
  if (he) std::memcpy(he, r->he.data(), r->he.size() * sizeof(int));
  if (he_v) std::memcpy(he_v, r->he_v.data(), r->he_v.size() * sizeof(int));
  if (he_f) std::memcpy(he_f, r->he_f.data(), r->he_f.size() * sizeof(int));
}

void ref_dmc_free(void* h) {
  auto* r = (DmcResult*)h;
  g_results.erase(std::remove(g_results.begin(), g_results.end(), r), g_results.end());
  delete r;
}

// Per-stage check: colours after colorFaces, and valences, for a given quad mesh with its
// inherited colours (cpp_dmc/DualMarchingCubes.cpp:714, :847).
void ref_dmc_color_valence(int nr_v, int nr_q, const int* quads, int* colors_inout, int* valence_out) {
  QuietStdout q;
  dmc::DualMarchingCubes d;
  std::vector<int> qv(quads, quads + 4 * (size_t)nr_q);
  std::vector<std::array<int, 5>> he;
  std::vector<int> hv, hf;
  d.halfedges(nr_v, qv, he, hv, hf);
  std::vector<int> col(colors_inout, colors_inout + nr_q);
  d.colorFaces(he, hf, col);
  std::copy(col.begin(), col.end(), colors_inout);
  std::vector<int> vv;
  d.vertexValence(nr_v, he, vv);
  std::copy(vv.begin(), vv.end(), valence_out);
}

// The DMC front end alone (before unused-vertex removal is folded in): quads and colours in
// map-key order, as collectQuadrilaterals (cpp_dmc/DualMarchingCubes.h:663) emits them.
void* ref_dmc_front(int nx, int ny, int nz, const double* origin, const double* spacing,
                    const float* field, double iso, int flip, int** colors_out, int* nr_colors) {
  QuietStdout q;
  dmc::UniformGrid ug;
  fill_grid(ug, nx, ny, nz, origin, spacing, field, flip);
  dmc::DualMarchingCubes d;
  auto* r = new DmcResult();
  std::vector<dmc::Vector> v, n;
  std::map<int, std::array<int, 5>> m_;
  for (int k = 0; k < nz - 1; k++)
    for (int j = 0; j < ny - 1; j++)
      for (int i = 0; i < nx - 1; i++) {
        double u[8];
        u[0] = ug.scalar(i, j, k); u[1] = ug.scalar(i + 1, j, k);
        u[2] = ug.scalar(i, j + 1, k); u[3] = ug.scalar(i + 1, j + 1, k);
        u[4] = ug.scalar(i, j, k + 1); u[5] = ug.scalar(i + 1, j, k + 1);
        u[6] = ug.scalar(i, j + 1, k + 1); u[7] = ug.scalar(i + 1, j + 1, k + 1);
        unsigned c = 0;
        for (int b = 0; b < 8; b++) c += ((unsigned)(u[b] >= iso)) << b;
        if (c == 0 || c == 255) continue;
        d.slice(iso, c, i, j, k, u, ug, v, n, m_);
      }
  std::vector<int> colors;
  d.collectQuadrilaterals(r->quads, colors, m_);
  d.removeUnusedVertices(v, n, r->quads);
  for (auto& p : v) { r->v.push_back(p[0]); r->v.push_back(p[1]); r->v.push_back(p[2]); }
  for (auto& p : n) { r->n.push_back(p[0]); r->n.push_back(p[1]); r->n.push_back(p[2]); }
  int* cc = (int*)std::malloc(sizeof(int) * (colors.size() + 1));
  std::copy(colors.begin(), colors.end(), cc);
  *colors_out = cc;
  *nr_colors = (int)colors.size();
  g_results.push_back(r);
  return r;
}

void ref_free_buffer(void* p) { std::free(p); }

}  // extern "C"
