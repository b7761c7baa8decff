// Implicit fields evaluated on the GPU: the reference's predefined test surfaces
// (p_mc::UniformGrid::generateVolume and its kernel, dmc/UniformGrid.cu:21-217; their formulas and
// constants define the test volumes, so they are kept as the reference has them), plus the two field
// families of the batched benchmark workload (a triply periodic field and a sum of Gaussian blobs).
// Points sit on [-1, 1]^3 at x = -1 + i * dx with the reference's float32 spacing dx = 2 / (n - 1),
// and every field is evaluated in float32, as the reference's generator does.
//
// One function serves the stored path (tmc_field_generate, a kernel that writes the field to
// memory) and the fused path (the classification evaluates the field instead of reading it), so
// both give the same values bit for bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tmc_gb300.h"

namespace tmc {

constexpr int kMaxBlobs = 16;

// Parameters of a generated field (device copy).
struct GenParams {
  int surface;           // TMC_SURF_*
  int count;             // TMC_SURF_BLOBS: blobs
  float k;               // TMC_SURF_PERIODIC: wave number
  float c[kMaxBlobs][3];  // blob centres
  float inv2s2[kMaxBlobs];  // 1 / (2 sigma^2)
  // fused path, separable surfaces (axis_separable): per-axis terms of every grid index, built by
  // axis_terms (so the values are those the stored path computes per point); null otherwise
  const float2* tab[3];
};

__device__ __forceinline__ float gsq(float x) { return x * x; }

// The surfaces that are sums and products of terms of one coordinate each, combined in the order
// the formula rounds them: the periodic field (sin and cos of k x), the reference's IWP, P-W hybrid
// and Neovius surfaces (cos of s (x + 1)), its sphere (x^2) and its Goursat surface (x^4, x^2).
__host__ __device__ __forceinline__ bool axis_separable(int surface) {
  return surface == TMC_SURF_PERIODIC || surface == TMC_SURF_IWP || surface == TMC_SURF_PW_HYBRID ||
         surface == TMC_SURF_NEOVIUS || surface == TMC_SURF_SPHERE || surface == TMC_SURF_GOURSAT;
}

// The per-axis terms of a separable surface at coordinate x: (sin kx, cos kx) for the periodic field,
// (cos s(x + 1), 0) for the cosine surfaces, (x^2, 0) for the sphere, (x^4, x^2) for Goursat's.
__device__ __forceinline__ float2 axis_terms(const GenParams& P, float x) {
  const float pi = 3.14159265358979323846f;
  switch (P.surface) {
    case TMC_SURF_PERIODIC:
      return make_float2(sinf(P.k * x), cosf(P.k * x));
    case TMC_SURF_IWP:
      return make_float2(cosf(5.01f * pi * (x + 1)), 0.0f);
    case TMC_SURF_PW_HYBRID:
      return make_float2(cosf(1.01f * pi * (x + 1)), 0.0f);
    case TMC_SURF_SPHERE:
      return make_float2(x * x, 0.0f);
    case TMC_SURF_GOURSAT:
      return make_float2(gsq(gsq(x)), x * x);
    default:  // TMC_SURF_NEOVIUS
      return make_float2(cosf(pi * (x + 1)), 0.0f);
  }
}

// A separable surface from its three per-axis terms
__device__ __forceinline__ float combine_terms(int surface, float2 X, float2 Y, float2 Z) {
  switch (surface) {
    case TMC_SURF_SPHERE:  // x^2 + y^2 + z^2 - 0.16
      return X.x + Y.x + Z.x - 0.16f;
    case TMC_SURF_GOURSAT: {  // x^4 + y^4 + z^4 - (x^2 + y^2 + z^2) + 0.5
      const float r2 = X.y + Y.y + Z.y;
      return X.x + Y.x + Z.x - r2 + 0.5f;
    }
    case TMC_SURF_PERIODIC:  // sin(kx)cos(ky) + sin(ky)cos(kz) + sin(kz)cos(kx)
      return X.x * Y.y + Y.x * Z.y + Z.x * X.y;
    case TMC_SURF_IWP: {
      const float cx = X.x, cy = Y.x, cz = Z.x;
      return cx * cy + cy * cz + cz * cx - cx * cy * cz;
    }
    case TMC_SURF_PW_HYBRID: {
      const float cx = X.x, cy = Y.x, cz = Z.x;
      return 4.0f * (cx * cy + cy * cz + cz * cx) - 3 * cx * cy * cz + 0.8f;
    }
    default: {  // TMC_SURF_NEOVIUS
      const float cx = X.x, cy = Y.x, cz = Z.x;
      return 3 * (cx + cy + cz) + 4 * cx * cy * cz;
    }
  }
}

// torus around the z axis (horizontal) or the y axis (vertical): ring radius R, tube radius r
__device__ __forceinline__ float torus_field(float x, float y, float z, float cx, float cy, float cz, bool vertical) {
  const float R2 = gsq(0.3f), r2 = gsq(0.15f);
  const float X = gsq(x - cx), Y = gsq(y - cy), Z = gsq(z - cz);
  return gsq(X + Y + Z + R2 - r2) - 4 * R2 * (X + (vertical ? Z : Y));
}

static __device__ __noinline__ float surface_value(const GenParams& P, float x, float y, float z) {
  const float pi = 3.14159265358979323846f;
  switch (P.surface) {
    case TMC_SURF_TORUS:
      return torus_field(x, y, z, 0, 0, 0, false);
    case TMC_SURF_TWO_HOLED_TORUS:
      return fminf(torus_field(x, y, z, -0.38f, 0, 0, false), torus_field(x, y, z, 0.2f, 0.38f, 0, false));
    case TMC_SURF_FOUR_HOLED_TORUS: {
      const float a = fminf(torus_field(x, y, z, -0.38f, 0, 0, false), torus_field(x, y, z, 0.38f, 0, 0, false));
      const float b = fminf(torus_field(x, y, z, 0, 0, -0.38f, true), torus_field(x, y, z, 0, 0, 0.38f, true));
      return fminf(a, b);
    }
    case TMC_SURF_IWP:
    case TMC_SURF_PW_HYBRID:
    case TMC_SURF_NEOVIUS:
    case TMC_SURF_PERIODIC:
    case TMC_SURF_SPHERE:
    case TMC_SURF_GOURSAT:
      return combine_terms(P.surface, axis_terms(P, x), axis_terms(P, y), axis_terms(P, z));
    case TMC_SURF_STEINER_ROMAN: {
      const float X = 1.5f * x, Y = 1.5f * y, Z = 1.5f * z;
      return gsq(X * X + Y * Y + Z * Z - 1.0f) - (gsq(Z - 1) - 2.0f * X * X) * (gsq(Z + 1) - 2 * Y * Y);
    }
    case TMC_SURF_BLOBS: {  // sum of exp(-|p - c|^2 / (2 sigma^2))
      float f = 0;
      for (int b = 0; b < P.count; b++) {
        const float d2 = gsq(x - P.c[b][0]) + gsq(y - P.c[b][1]) + gsq(z - P.c[b][2]);
        f += expf(-d2 * P.inv2s2[b]);
      }
      return f;
    }
    default: {  // TMC_SURF_GENUS_TWO: the domain mapped to [-2, 2]^3
      const float X = 4.0f * ((x + 1.0f) / 2.0f) - 2.0f;
      const float Y = 4.0f * ((y + 1.0f) / 2.0f) - 2.0f;
      const float Z = 4.0f * ((z + 1.0f) / 2.0f) - 2.0f;
      float t = 2 * Y * (Y * Y - 3 * X * X) * (1 - Z * Z);
      t += (X * X + Y * Y) * (X * X + Y * Y);
      t -= (9 * Z * Z - 1) * (1 - Z * Z);
      return t;
    }
  }
}

// The value at grid point (i, j, k): coordinates -1 + i * dx in float32, as the reference forms them.
__device__ __forceinline__ float generated_at(const GenParams& P, const float d[3], int i, int j, int k) {
  return surface_value(P, -1.0f + i * d[0], -1.0f + j * d[1], -1.0f + k * d[2]);
}

// Per-axis tables of a separable surface: tab[a][i] = axis_terms at the i-th coordinate of axis a
// (the three axes one after another, n[a] entries each).
static __global__ void axis_terms_kernel(GenParams P, int nx, int ny, int nz, float dx, float dy, float dz, float2* out) {
  const int total = nx + ny + nz;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    const int a = q < nx ? 0 : (q < nx + ny ? 1 : 2);
    const int i = q - (a == 0 ? 0 : (a == 1 ? nx : nx + ny));
    const float d = a == 0 ? dx : (a == 1 ? dy : dz);
    out[q] = axis_terms(P, -1.0f + i * d);
  }
}

// Host side: parameters and spacing of a generator, checked.  Returns false for a bad descriptor.
inline bool gen_params(const tmc_generator& s, GenParams& P, float d[3]) {
  if (s.surface < TMC_SURF_SPHERE || s.surface > TMC_SURF_BLOBS) return false;
  if (s.nx < 2 || s.ny < 2 || s.nz < 2 || s.nx > 65535 || s.ny > 65535 || s.nz > 65535) return false;
  P = GenParams{};
  P.surface = s.surface;
  if (s.surface == TMC_SURF_PERIODIC) {
    P.k = (float)s.params[0];
    if (!(P.k == P.k) || P.k > 1e30f || P.k < -1e30f) return false;
  }
  if (s.surface == TMC_SURF_BLOBS) {
    if (s.count < 1 || s.count > kMaxBlobs) return false;
    P.count = s.count;
    for (int b = 0; b < s.count; b++) {
      const double sig = s.params[4 * b + 3];
      if (!(sig > 0) || sig > 1e30) return false;
      for (int a = 0; a < 3; a++) P.c[b][a] = (float)s.params[4 * b + a];
      P.inv2s2[b] = (float)(1.0 / (2.0 * sig * sig));
    }
  }
  // the reference's spacing, in float32: (xmax - xmin) / (n - 1.0f)
  d[0] = 2.0f / (s.nx - 1.0f);
  d[1] = 2.0f / (s.ny - 1.0f);
  d[2] = 2.0f / (s.nz - 1.0f);
  return true;
}

}  // namespace tmc
