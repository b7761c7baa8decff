// DMC vertex representative (cpp_dmc/DualMarchingCubes.cpp:194-326), two implementations that
// return bit-identical results:
//
//  * representative_exact: the reference's mixed float/double arithmetic restated line by line in
//    float64 (each float64 operation rounded on its own: the library is built with -fmad=false).
//  * representative_fast: the same decisions and outputs, computed on the FP32 pipes.  All 7x7
//    samples are first evaluated in float32 with rigorous error bounds; only the samples that can
//    still be the argmin (their distance interval overlaps the best certain one) are evaluated
//    exactly, with float-float arithmetic and certified rounding (ffloat.cuh).  Any rounding that
//    cannot be certified sends the projection to the float64 path.
//
// Host + device: tests/cpp/repr_check.cpp runs both on the CPU against the oracle.
#pragma once
#include <cmath>
#include <cstdint>

#include "ffloat.cuh"

namespace tmc {
namespace repr {

using ffx::ff;

TMC_HD int nibr(uint64_t w, int i) { return (int)((w >> (4 * i)) & 0xF); }

// contour packing as in common.cuh: nibbles 0..11 edges, 12..15 sizes
TMC_HD int csize(uint64_t c, int t) { return nibr(c, 12 + t); }
TMC_HD int ccount(uint64_t c) { return (csize(c, 0) > 0) + (csize(c, 1) > 0) + (csize(c, 2) > 0) + (csize(c, 3) > 0); }
TMC_HD int cedge(uint64_t c, int flat) { return nibr(c, flat); }

// edge end vertices and axis / lower-corner offset (same packing as mc_tables.h)
constexpr uint64_t EDGE_V0 = 0x231046540210ull;
constexpr uint64_t EDGE_V1 = 0x675467752331ull;
constexpr uint64_t EDGE_AXIS = 0x222210101010ull;

struct Boxes {
  float b[4][3][2];  // contour, axis, min/max
};

struct Stats {
  int fail1 = 0, fail2 = 0;  // 7x7 projection found nothing / 26x26 neither (the reference's counters)
  int fallback = 0;          // sample values that needed float64
  int normal_f64 = 0;        // normals computed in float64 (strong cancellation)
};

// ---------------------------------------------------------------------------------------------
// edge parameter: getLocalCoordinates (cpp_dmc/DualMarchingCubes.h:391-407), l rounded to float
// ---------------------------------------------------------------------------------------------
// the reference's float64 parameter; the two corner values are passed by value (a pointer would
// force the caller's corners into local memory)
TMC_HD_COLD float edge_param_f64(double iso, float f0, float f1) {
  return (float)((iso - (double)f0) / ((double)f1 - (double)f0));
}
TMC_HD float edge_param_exact(int e, const float u[8], double iso) {
  const int v0 = nibr(EDGE_V0, e), v1 = nibr(EDGE_V1, e);
  return edge_param_f64(iso, u[v0], u[v1]);
}

// corner value v of the eight (selects: a run-time index keeps u in registers)
TMC_HD float corner_at(const float u[8], int v) {
  float r = u[0];
#pragma unroll
  for (int q = 1; q < 8; q++) r = (v == q) ? u[q] : r;
  return r;
}

TMC_HD float edge_param_fast(int e, const float u[8], double iso, ff iso_ff, bool& fallback) {
  const int v0 = nibr(EDGE_V0, e), v1 = nibr(EDGE_V1, e);
  const float f0 = corner_at(u, v0), f1 = corner_at(u, v1);
  const ff num = ffx::ff_sub(iso_ff, ffx::ff_from(f0));
  const ff den = ffx::two_sum(f1, -f0);  // exact
  const ff q = ffx::ff_div(num, den);
  const float aq = fabsf(q.hi);
  const float mag = fmaxf(fabsf(iso_ff.hi), fabsf(f0));
  const float err = aq * 0x1p-42f + mag * 0x1p-45f / fabsf(den.hi);
  float l;
  if (ffx::ff_round(q, err, l)) return l;
  fallback = true;
  return edge_param_f64(iso, f0, f1);
}

// local coordinates of the crossing on edge e: l * val + con in float, as the reference
TMC_HD void local_from_param(int e, float l, float out[3]) {
  const int ax = nibr(EDGE_AXIS, e), con = nibr(EDGE_V0, e);
  for (int d = 0; d < 3; d++) {
    const float val = (d == ax) ? 1.0f : 0.0f;
    const float cn = (float)((con >> d) & 1);
    out[d] = l * val + cn;
  }
}

// ---------------------------------------------------------------------------------------------
// exact float64 path (cpp_dmc/DualMarchingCubes.cpp:194-326)
// ---------------------------------------------------------------------------------------------
TMC_HD bool in_neighbor_bbox(double u, double v, double w, uint64_t c, int t, const Boxes& bx, int A, int B, int W) {
  const int n = ccount(c);
  for (int i = 0; i < n; i++) {
    if (csize(c, i) == 3 && t != i) {
      if (u < (double)bx.b[i][A][0] || (double)bx.b[i][A][1] < u) continue;
      if (v < (double)bx.b[i][B][0] || (double)bx.b[i][B][1] < v) continue;
      if (w < (double)bx.b[i][W][0] || (double)bx.b[i][W][1] < w) continue;
      return true;
    }
  }
  return false;
}

TMC_HD bool projection_exact(const double fp[8], double iso, uint64_t c, int t, double p[3], const Boxes& bx, int A,
                        int B, int W, int nrSamples) {
  const double umin = bx.b[t][A][0], umax = bx.b[t][A][1];
  const double vmin = bx.b[t][B][0], vmax = bx.b[t][B][1];
  const double du = (umax - umin) / (nrSamples - 1);
  const double dv = (vmax - vmin) / (nrSamples - 1);
  double minDistance = 100;
  double pt0 = 0, pt1 = 0, pt2 = -1;
  double wmin = bx.b[t][W][0], wmax = bx.b[t][W][1];
  const double eps = 1e-5;
  if (fabs(wmax - wmin) < eps) {
    wmin -= eps;
    wmax += eps;
  }
  const int cnt = ccount(c);
  const int cnt_sz = csize(c, t);
  for (int i = 1; i < (nrSamples - 1); i++) {
    const float u = umin + i * du;
    for (int j = 1; j < (nrSamples - 1); j++) {
      const float v = vmin + j * dv;
      const float g1 = (1 - v) * ((1 - u) * fp[0] + u * fp[1]) + v * ((1 - u) * fp[2] + u * fp[3]);
      const float g2 = (1 - v) * ((1 - u) * fp[4] + u * fp[5]) + v * ((1 - u) * fp[6] + u * fp[7]);
      if (g1 == g2) continue;
      const float w = (iso - g1) / (g2 - g1);
      if (wmin <= w && w <= wmax) {
        if (cnt == 1 || cnt_sz == 3 || !in_neighbor_bbox(u, v, w, c, t, bx, A, B, W)) {
          const float d = (p[0] - u) * (p[0] - u) + (p[1] - v) * (p[1] - v) + (p[2] - w) * (p[2] - w);
          if (minDistance > d) {
            minDistance = d;
            pt0 = u;
            pt1 = v;
            pt2 = w;
          }
        }
      }
    }
  }
  if (pt2 > -1) {
    p[0] = pt0;
    p[1] = pt1;
    p[2] = pt2;
    return true;
  }
  return false;
}

// plane axes (A, B, W) and corner permutation of the three projection planes (w_proj, v_proj,
// u_proj, cpp_dmc/DualMarchingCubes.cpp:198-200)
TMC_HD void plane(int prj, int& A, int& B, int& W, uint32_t& perm) {
  if (prj == 0) { A = 0; B = 1; W = 2; perm = 0x76543210u; }
  else if (prj == 1) { A = 0; B = 2; W = 1; perm = 0x76325410u; }
  else { A = 1; B = 2; W = 0; perm = 0x75316420u; }
}

// projection plane from the trilinear gradient at p (contours of 6 or more edges)
TMC_HD int plane_from_gradient(const double f[8], const double p[3]) {
  const double uu = p[0], vv = p[1], ww = p[2];
  const double g0 = (1 - ww) * ((1 - vv) * (f[1] - f[0]) + vv * (f[3] - f[2])) + ww * ((1 - vv) * (f[5] - f[4]) + vv * (f[7] - f[6]));
  const double g1 = (1 - ww) * ((1 - uu) * (f[2] - f[0]) + uu * (f[3] - f[1])) + ww * ((1 - uu) * (f[6] - f[4]) + uu * (f[7] - f[5]));
  const double g2 = (1 - vv) * ((1 - uu) * (f[4] - f[0]) + uu * (f[5] - f[1])) + vv * ((1 - uu) * (f[6] - f[2]) + uu * (f[7] - f[3]));
  const double dx = fabs(g0), dy = fabs(g1), dz = fabs(g2);
  if (dz >= dx && dz >= dy) return 0;
  if (dy >= dx && dy >= dz) return 1;
  if (dx >= dy && dx >= dz) return 2;
  return 0;
}

// projection plane from the bounding-box extents (minProjection)
TMC_HD int plane_from_extent(const Boxes& bx, int t) {
  const double su = (double)bx.b[t][0][1] - (double)bx.b[t][0][0];
  const double sv = (double)bx.b[t][1][1] - (double)bx.b[t][1][0];
  const double sw = (double)bx.b[t][2][1] - (double)bx.b[t][2][0];
  if (sw <= su && sw <= sv) return 0;
  if (sv <= su && sv <= sw) return 1;
  if (su <= sv && su <= sw) return 2;
  return 0;
}

// the contour's mean point exactly as the reference accumulates it (float64)
struct Point64 {
  double p[3];
};
TMC_HD_COLD Point64 mean_point_exact(const float* pts, int n) {
  Point64 r;
  r.p[0] = r.p[1] = r.p[2] = 0;
  for (int q = 0; q < n; q++) {
    r.p[0] += pts[3 * q];
    r.p[1] += pts[3 * q + 1];
    r.p[2] += pts[3 * q + 2];
  }
  r.p[0] /= n;
  r.p[1] /= n;
  r.p[2] /= n;
  return r;
}

// representative with the projection from `prj`; p in: mean point, out: representative
TMC_HD void representative_exact_plane(const float u[8], double iso, uint64_t c, int t, double p[3], const Boxes& bx,
                                       int prj, Stats& st) {
  double f[8];
  for (int q = 0; q < 8; q++) f[q] = u[q];
  int A, B, W;
  uint32_t perm;
  plane(prj, A, B, W, perm);
  double fp[8];
  for (int q = 0; q < 8; q++) fp[q] = f[(perm >> (4 * q)) & 0xF];
  double pt[3] = {p[A], p[B], p[W]};
  if (!projection_exact(fp, iso, c, t, pt, bx, A, B, W, 9)) {
    st.fail1++;
    if (!projection_exact(fp, iso, c, t, pt, bx, A, B, W, 28)) st.fail2++;
  }
  p[A] = pt[0];
  p[B] = pt[1];
  p[W] = pt[2];
}

TMC_HD void representative_exact(const float u[8], double iso, uint64_t c, int t, double p[3], const Boxes& bx,
                                 Stats& st) {
  int prj;
  if (csize(c, t) >= 6) {
    double f[8];
    for (int q = 0; q < 8; q++) f[q] = u[q];
    prj = plane_from_gradient(f, p);
  } else {
    prj = plane_from_extent(bx, t);
  }
  representative_exact_plane(u, iso, c, t, p, bx, prj, st);
}

// ---------------------------------------------------------------------------------------------
// fast path
// ---------------------------------------------------------------------------------------------
// Corner values passed by value to out-of-line helpers (the caller's copy stays in registers).
struct Corners {
  float f[8];
};

struct SampleApprox {
  float D, ED;
  int status;  // 0 invalid, 1 valid, 2 uncertain
};

// Projection state: scalar fields and constant-indexed arrays only, so that it lives in registers.
struct ProjCtx {
  float fp[8];             // permuted corner values
  float wlo, whi;          // w >= wlo && w <= whi  <=>  wmin <= w <= wmax (double bounds)
  float pf[3];             // mean point (approximate, |error| <= 2^-23)
  ff pff[3];               // mean point (float-float, within 2^-43 of the reference's double)
  float iso_f;
  float iso_err;           // |iso - iso_f|
  ff iso_ff;
  double iso_d;
  float sabs_lo, sabs_hi;  // max |f| over the w = 0 and the w = 1 face (bounds of the bilinear sums)
  bool excl;               // the neighbour-contour exclusion applies (more than one contour, size != 3)
  int cnt, t, A, B, W;
  uint64_t c;
  const Boxes* bx;
};

// float32 evaluation of one sample with error bounds.  With u, v in [0, 1] the bilinear weights
// are in [0, 1] and sum to 1, so every partial sum is bounded by the face's max |f|.
TMC_HD SampleApprox sample_approx(const ProjCtx& P, float u, float v) {
  SampleApprox r;
  const float omu = 1 - u, omv = 1 - v;
  const float* f = P.fp;
  const float A1 = ffx::fma_rn(u, f[1], omu * f[0]), B1 = ffx::fma_rn(u, f[3], omu * f[2]);
  const float A2 = ffx::fma_rn(u, f[5], omu * f[4]), B2 = ffx::fma_rn(u, f[7], omu * f[6]);
  const float g1 = ffx::fma_rn(v, B1, omv * A1), g2 = ffx::fma_rn(v, B2, omv * A2);
  const float Eg1 = P.sabs_lo * 0x1p-20f + fabsf(g1) * 0x1p-23f;
  const float Eg2 = P.sabs_hi * 0x1p-20f + fabsf(g2) * 0x1p-23f;
  const float den = g2 - g1;
  const float Eden = (Eg1 + Eg2 + fabsf(den) * 0x1p-23f) * 1.0001f;
  if (!(fabsf(den) > 2 * Eden)) {  // w unknown (includes g1 == g2)
    r.D = 0;
    r.ED = INFINITY;
    r.status = 2;
    return r;
  }
  const float num = P.iso_f - g1;
  const float Enum = Eg1 + P.iso_err + fabsf(num) * 0x1p-23f;
  const float w = num / den;
  const float aw = fabsf(w);
  const float Ew = ((Enum + aw * Eden) / (fabsf(den) - Eden) + aw * 0x1p-21f) * 1.0001f + 1e-30f;
  // range check
  const bool sure_in = (w - Ew >= P.wlo) && (w + Ew <= P.whi);
  const bool sure_out = (w + Ew < P.wlo) || (w - Ew > P.whi);
  int status = sure_out ? 0 : (sure_in ? 1 : 2);
  if (status != 0 && P.excl) {
    for (int i = 0; i < P.cnt; i++) {
      if (csize(P.c, i) == 3 && P.t != i) {
        const Boxes& bx = *P.bx;
        if (u < bx.b[i][P.A][0] || bx.b[i][P.A][1] < u) continue;
        if (v < bx.b[i][P.B][0] || bx.b[i][P.B][1] < v) continue;
        const float lo = bx.b[i][P.W][0], hi = bx.b[i][P.W][1];
        if (w + Ew < lo || w - Ew > hi) continue;  // surely outside this box
        if (w - Ew >= lo && w + Ew <= hi) {        // surely inside: excluded
          status = 0;
          break;
        }
        status = 2;  // may be excluded
      }
    }
  }
  r.status = status;
  const float e0 = P.pf[0] - u, e1 = P.pf[1] - v, e2 = P.pf[2] - w;
  const float D = e0 * e0 + e1 * e1 + e2 * e2;
  const float Ep = 0x1p-22f;
  r.D = D;
  r.ED = (2 * (fabsf(e0) + fabsf(e1)) * Ep + 2 * fabsf(e2) * (Ew + Ep) + (Ew + Ep) * (Ew + Ep) + 2 * Ep * Ep +
          D * 0x1p-20f) * 1.0001f + 1e-30f;
  return r;
}

// One exactly evaluated sample, returned by value.
struct SampleOut {
  float w, d;
  int status;  // 0 invalid, 1 valid, 2 distance rounding not certified (evaluate in float64)
  int f64;     // values recomputed in float64
};

// The reference's bilinear value of one face at (u, v), float64 rounded to float (its (1 - u) is a
// float subtraction, cpp_dmc/DualMarchingCubes.cpp:302-303).  Used where the float-float value lies
// on (or within its error of) a float rounding midpoint, e.g. exact ties at dyadic samples.
TMC_HD_COLD float bilinear_f64(float f0, float f1, float f2, float f3, float u, float v) {
  const float omu = 1 - u, omv = 1 - v;
  return (float)((double)omv * ((double)omu * f0 + (double)u * f1) + (double)v * ((double)omu * f2 + (double)u * f3));
}
// the reference's w = (iso - g1) / (g2 - g1): float64 over the float difference (:305)
TMC_HD_COLD float w_f64(double iso, float g1, float g2) {
  const float den = g2 - g1;
  return (float)((iso - (double)g1) / (double)den);
}

// float64 evaluation of one sample, as the reference's loop body (projection, :298-316).  Rare:
// out of line, with the context copied (the caller's stays in registers).
TMC_HD_COLD SampleOut sample_f64(const ProjCtx P, double pd0, double pd1, double pd2, float u, float v) {
  SampleOut r{0.0f, 0.0f, 0};
  double fp[8];
  for (int q = 0; q < 8; q++) fp[q] = P.fp[q];
  const float g1 = (1 - v) * ((1 - u) * fp[0] + u * fp[1]) + v * ((1 - u) * fp[2] + u * fp[3]);
  const float g2 = (1 - v) * ((1 - u) * fp[4] + u * fp[5]) + v * ((1 - u) * fp[6] + u * fp[7]);
  if (g1 == g2) return r;
  const float w = (P.iso_d - g1) / (g2 - g1);
  if (!(w >= P.wlo && w <= P.whi)) return r;
  if (P.excl && in_neighbor_bbox(u, v, w, P.c, P.t, *P.bx, P.A, P.B, P.W)) return r;
  r.status = 1;
  r.w = w;
  r.d = (pd0 - u) * (pd0 - u) + (pd1 - v) * (pd1 - v) + (pd2 - w) * (pd2 - w);
  return r;
}

// exact evaluation of one sample (status 2 when a rounding cannot be certified)
TMC_HD SampleOut sample_exact(const ProjCtx& P, float u, float v) {
  SampleOut r{0.0f, 0.0f, 2, 0};
  const float omu = 1 - u, omv = 1 - v;
  const float* f = P.fp;
  const ff A1 = ffx::ff_add(ffx::two_prod(omu, f[0]), ffx::two_prod(u, f[1]));
  const ff B1 = ffx::ff_add(ffx::two_prod(omu, f[2]), ffx::two_prod(u, f[3]));
  const ff A2 = ffx::ff_add(ffx::two_prod(omu, f[4]), ffx::two_prod(u, f[5]));
  const ff B2 = ffx::ff_add(ffx::two_prod(omu, f[6]), ffx::two_prod(u, f[7]));
  const ff G1 = ffx::ff_add(ffx::ff_mul_f(A1, omv), ffx::ff_mul_f(B1, v));
  const ff G2 = ffx::ff_add(ffx::ff_mul_f(A2, omv), ffx::ff_mul_f(B2, v));
  // |G - the reference's float64 value| <= ~2^-45 * (|1-v| |A| + |v| |B|): the float-float
  // operations' relative errors on these magnitudes plus the reference's own float64 roundings
  const float S1 = fabsf(omv) * fabsf(A1.hi) + fabsf(v) * fabsf(B1.hi);
  const float S2 = fabsf(omv) * fabsf(A2.hi) + fabsf(v) * fabsf(B2.hi);
  float g1, g2;
  if (!ffx::ff_round(G1, S1 * 0x1p-44f, g1)) {
    g1 = bilinear_f64(f[0], f[1], f[2], f[3], u, v);
    r.f64++;
  }
  if (!ffx::ff_round(G2, S2 * 0x1p-44f, g2)) {
    g2 = bilinear_f64(f[4], f[5], f[6], f[7], u, v);
    r.f64++;
  }
  if (g1 == g2) {
    r.status = 0;
    return r;
  }
  const float den = g2 - g1;  // the reference subtracts the two floats
  const ff num = ffx::ff_sub(P.iso_ff, ffx::ff_from(g1));
  const ff W = ffx::ff_div(num, ffx::ff_from(den));
  const float errW = fabsf(W.hi) * 0x1p-42f + (fabsf(P.iso_ff.hi) * 0x1p-46f + fabsf(num.hi) * 0x1p-50f) / fabsf(den);
  float w;
  if (!ffx::ff_round(W, errW, w)) {
    w = w_f64(P.iso_d, g1, g2);
    r.f64++;
  }
  bool valid = (w >= P.wlo && w <= P.whi);
  if (valid && P.excl) {
    const Boxes& bx = *P.bx;
    for (int i = 0; i < P.cnt; i++) {
      if (csize(P.c, i) == 3 && P.t != i) {
        if (u < bx.b[i][P.A][0] || bx.b[i][P.A][1] < u) continue;
        if (v < bx.b[i][P.B][0] || bx.b[i][P.B][1] < v) continue;
        if (w < bx.b[i][P.W][0] || bx.b[i][P.W][1] < w) continue;
        valid = false;
        break;
      }
    }
  }
  if (!valid) {
    r.status = 0;
    return r;
  }
  const ff d0 = ffx::ff_sub(P.pff[0], ffx::ff_from(u));
  const ff d1 = ffx::ff_sub(P.pff[1], ffx::ff_from(v));
  const ff d2 = ffx::ff_sub(P.pff[2], ffx::ff_from(w));
  const ff D = ffx::ff_add(ffx::ff_add(ffx::ff_mul(d0, d0), ffx::ff_mul(d1, d1)), ffx::ff_mul(d2, d2));
  const float errD = fabsf(D.hi) * 0x1p-40f + (fabsf(d0.hi) + fabsf(d1.hi) + fabsf(d2.hi)) * 0x1p-41f;
  float d;
  if (!ffx::ff_round(D, errD, d)) return r;
  r.w = w;
  r.d = d;
  r.status = 1;
  return r;
}

// u_i = fl32(umin + i*(umax-umin)/8) as the reference computes it in float64, for i = 1..7.
// Both ends are floats in [0, 1].  When their exponents differ by at most 20 (or lo is 0), the
// float64 computation is exact (at most 24+20+3 significant bits), so the reference rounds the
// exact value once; the float-float sum is exact too and its high part is that rounding.
// Otherwise the value is certified, and computed in float64 when that fails.
TMC_HD_COLD float sample_coord_f64(float lo, float hi, int i) {
  const double du = ((double)hi - (double)lo) / 8;
  return (float)((double)lo + i * du);
}
TMC_HD void sample_coords(float lo, float hi, float out[7], int& f64_count) {
  const ff D = ffx::two_sum(hi, -lo);  // exact difference
  const int ehi = (int)((ffx::fbits(hi) >> 23) & 0xFF), elo = (int)((ffx::fbits(lo) >> 23) & 0xFF);
  const bool exact = (lo == 0.0f) || (hi == lo) || (ehi - elo <= 20 && elo > 0);
  // not unrolled: the set-up pass writes `out` straight into its record in global memory, and
  // one copy of the body keeps the pass's code small (it is bound by instruction fetch)
#pragma unroll 1
  for (int i = 1; i <= 7; i++) {
    const ff a = ffx::two_prod((float)i, D.hi);
    const ff b = ffx::two_prod((float)i, D.lo);
    ff s = ffx::ff_add(a, b);
    s.hi *= 0.125f;
    s.lo *= 0.125f;
    const ff x = ffx::ff_add(ffx::ff_from(lo), s);
    if (exact) {
      out[i - 1] = x.hi;
      continue;
    }
    const float err = (fabsf(lo) + fabsf(s.hi)) * 0x1p-44f;
    if (!ffx::ff_round(x, err, out[i - 1])) {
      out[i - 1] = sample_coord_f64(lo, hi, i);
      f64_count++;
    }
  }
}

// index of the coordinate nearest to x (the first on ties)
TMC_HD int nearest_sample(const float s[7], float x) {
  int k = 0;
  float best = fabsf(s[0] - x);
#pragma unroll 1
  for (int q = 1; q < 7; q++) {
    const float d = fabsf(s[q] - x);
    if (d < best) {
      best = d;
      k = q;
    }
  }
  return k;
}

// Evaluates sample (i, j) in float32: records the lower bound of its distance (+inf when it is
// surely invalid) and lowers m, the smallest certain upper bound of a valid sample's distance.
TMC_HD void approx_into(const ProjCtx& P, const float* us, const float* vs, int i, int j, float* buf, int stride,
                        float& m) {
  const SampleApprox s = sample_approx(P, us[i], vs[j]);
  if (s.status == 1) m = fminf(m, s.D + s.ED);
  buf[(7 * i + j) * stride] = (s.status == 0) ? INFINITY : s.D - s.ED;
}

// w window from the box's w extent, as the reference widens it (wmin -= 1e-5, wmax += 1e-5 when
// the extent is below 1e-5), as the float range [wlo, whi] of values inside the float64 window.
struct Window {
  float lo, hi;
};
TMC_HD_COLD Window w_window_flat(float lo, float hi) {
  double wmin = lo, wmax = hi;
  if (fabs(wmax - wmin) < 1e-5) {
    wmin -= 1e-5;
    wmax += 1e-5;
  }
  return Window{ffx::f_ceil(wmin), ffx::f_floor(wmax)};
}
TMC_HD void w_window(float lo, float hi, float& wlo, float& whi) {
  const float ext = hi - lo;  // within one ulp of the exact extent
  if (ext > 1.001e-5f) {      // surely not flat: the window is the box itself
    wlo = lo;
    whi = hi;
    return;
  }
  const Window w = w_window_flat(lo, hi);
  wlo = w.lo;
  whi = w.hi;
}

// index of the lowest set bit of a non-zero mask
TMC_HD int lowest_bit(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __ffsll((long long)x) - 1;
#else
  return __builtin_ctzll(x);
#endif
}

// 0 = found (pt set), 1 = no valid sample.  buf: 49 slots (lower bound of each sample's distance,
// +inf when it cannot win), slot q at buf[q * stride] (shared memory on the GPU, one column per
// thread).  The 3x3 samples around the mean point are approximated first; every other sample is
// skipped when even its distance within the sample plane exceeds the best certain bound (its w
// cannot make it smaller).  The surviving candidates are then evaluated exactly in the reference's
// loop order, so that ties resolve as the reference's strict `minDistance > d`.
// F64: evaluate uncertified samples in float64 (needs the contour points); otherwise return 2 at the
// first such sample.
template <bool F64 = true>
TMC_HD int projection_fast(const ProjCtx& P, const float* us, const float* vs, float pt[3], float* buf, int stride,
                           int& f64_samples, const float* pts, int npts) {
  float m = INFINITY;
  uint64_t done = 0;
  const int i0 = nearest_sample(us, P.pf[0]), j0 = nearest_sample(vs, P.pf[1]);
  const int ia = i0 > 0 ? i0 - 1 : 0, ib = i0 < 6 ? i0 + 1 : 6;
  const int ja = j0 > 0 ? j0 - 1 : 0, jb = j0 < 6 ? j0 + 1 : 6;
#pragma unroll 1
  for (int i = ia; i <= ib; i++)
#pragma unroll 1
    for (int j = ja; j <= jb; j++) {
      approx_into(P, us, vs, i, j, buf, stride, m);
      done |= 1ull << (7 * i + j);
    }
  // every other sample: skipped when even its distance within the sample plane (a lower bound of
  // the reference's float distance, whatever w is) exceeds m.  The samples that survive the bound
  // of the 3x3 seeds form a mask, taken lowest first so that the lanes of a warp evaluate their
  // k-th survivors together; m keeps falling meanwhile, so each is checked again before its turn.
  const float Ep = 0x1p-22f;
  float e1s[7];
#pragma unroll
  for (int j = 0; j < 7; j++) {
    const float e1 = fmaxf(fabsf(P.pf[1] - vs[j]) - Ep, 0.0f);
    e1s[j] = e1 * e1;
  }
  uint64_t need = 0;
#pragma unroll 1
  for (int i = 0; i < 7; i++) {
    const float e0 = fmaxf(fabsf(P.pf[0] - us[i]) - Ep, 0.0f);
#pragma unroll
    for (int j = 0; j < 7; j++) {
      const int q = 7 * i + j;
      if ((done >> q) & 1) continue;
      if ((e0 * e0 + e1s[j]) * (1.0f - 0x1p-20f) > m) buf[q * stride] = INFINITY;
      else need |= 1ull << q;
    }
  }
#pragma unroll 1
  while (need) {
    const int q = lowest_bit(need);
    need &= need - 1;
    const int i = q / 7, j = q - 7 * i;
    const float e0 = fmaxf(fabsf(P.pf[0] - us[i]) - Ep, 0.0f);
    const float e1 = fmaxf(fabsf(P.pf[1] - vs[j]) - Ep, 0.0f);
    if ((e0 * e0 + e1 * e1) * (1.0f - 0x1p-20f) > m) {
      buf[q * stride] = INFINITY;
      continue;
    }
    approx_into(P, us, vs, i, j, buf, stride, m);
  }
  // exact evaluation of every sample that can still win, in the reference's loop order.  The
  // candidates come from a bit mask, lowest first: the lanes of a warp then evaluate their k-th
  // candidates together instead of one loop slot at a time (a slot is rarely everyone's candidate).
  uint64_t cand = 0;
#pragma unroll 1
  for (int q = 0; q < 49; q++)
    if (buf[q * stride] <= m) cand |= 1ull << q;
  float best = 100.0f;
  bool found = false;
  bool have_pd = false;
  double pd[3] = {0, 0, 0};
#pragma unroll 1
  while (cand) {
    const int q = lowest_bit(cand);
    cand &= cand - 1;
    const int i = q / 7, j = q - 7 * i;
    SampleOut s = sample_exact(P, us[i], vs[j]);
    f64_samples += s.f64;
    if (s.status == 2) {
      if (!F64) return 2;
      if (!have_pd) {
        const Point64 pm = mean_point_exact(pts, npts);
        pd[0] = pm.p[P.A];
        pd[1] = pm.p[P.B];
        pd[2] = pm.p[P.W];
        have_pd = true;
      }
      s = sample_f64(P, pd[0], pd[1], pd[2], us[i], vs[j]);
      f64_samples++;
    }
    if (s.status != 1) continue;
    if (best > s.d) {
      best = s.d;
      pt[0] = us[i];
      pt[1] = vs[j];
      pt[2] = s.w;
      found = true;
    }
  }
  return found ? 0 : 1;
}

// exact comparison a <= b of two normalised float pairs
TMC_HD bool ff_le(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }

// the exact difference (s, e) of two floats is a float64 value (the reference's subtraction does
// not round) when its bits span at most 53 places
TMC_HD bool exact_in_f64(ff x) {
  if (x.lo == 0.0f) return true;
  const int es = (int)((ffx::fbits(x.hi) >> 23) & 0xFF), ee = (int)((ffx::fbits(x.lo) >> 23) & 0xFF);
  return ee > 0 && es - ee <= 29;
}

// projection plane from the box extents (minProjection).  The extents are float differences, held
// exactly as float pairs; when the reference's float64 subtractions are exact too the comparison
// is exact, otherwise (-1) it is redone in float64.
TMC_HD int plane_from_extent_box_ff(const float b[3][2]) {
  const ff su = ffx::two_sum(b[0][1], -b[0][0]);
  const ff sv = ffx::two_sum(b[1][1], -b[1][0]);
  const ff sw = ffx::two_sum(b[2][1], -b[2][0]);
  if (!exact_in_f64(su) || !exact_in_f64(sv) || !exact_in_f64(sw)) return -1;
  if (ff_le(sw, su) && ff_le(sw, sv)) return 0;
  if (ff_le(sv, su) && ff_le(sv, sw)) return 1;
  if (ff_le(su, sv) && ff_le(su, sw)) return 2;
  return 0;
}

// projection plane from the trilinear gradient at the mean point (contours of 6 or more edges),
// decided in float32 when no comparison is within its error bound, else in float64 (-1)
TMC_HD int plane_from_gradient_f(const float f[8], float uu, float vv, float ww) {
  const float a0 = f[1] - f[0], a1 = f[3] - f[2], a2 = f[5] - f[4], a3 = f[7] - f[6];
  const float b0 = f[2] - f[0], b1 = f[3] - f[1], b2 = f[6] - f[4], b3 = f[7] - f[5];
  const float c0 = f[4] - f[0], c1 = f[5] - f[1], c2 = f[6] - f[2], c3 = f[7] - f[3];
  const float g0 = (1 - ww) * ((1 - vv) * a0 + vv * a1) + ww * ((1 - vv) * a2 + vv * a3);
  const float g1 = (1 - ww) * ((1 - uu) * b0 + uu * b1) + ww * ((1 - uu) * b2 + uu * b3);
  const float g2 = (1 - vv) * ((1 - uu) * c0 + uu * c1) + vv * ((1 - uu) * c2 + uu * c3);
  float m = 0;
  for (int q = 0; q < 8; q++) m = fmaxf(m, fabsf(f[q]));
  // each |g| is within 2^-18 * max|f| of the reference's (weights in [0, 1], a dozen roundings and
  // the mean point within 2^-22)
  const float e = m * 0x1p-18f;
  const float dx = fabsf(g0), dy = fabsf(g1), dz = fabsf(g2);
  auto sure = [&](float a, float b) { return fabsf(a - b) > 2 * e; };  // a >= b decided
  if (!sure(dz, dx) || !sure(dz, dy) || !sure(dy, dx)) return -1;
  if (dz >= dx && dz >= dy) return 0;
  if (dy >= dx && dy >= dz) return 1;
  if (dx >= dy && dx >= dz) return 2;
  return 0;
}
TMC_HD int plane_from_extent_ff(const Boxes& bx, int t) { return plane_from_extent_box_ff(bx.b[t]); }
struct Box3 {
  float b[3][2];
};
TMC_HD_COLD int plane_from_extent_box_f64(Box3 x) {
  const double su = (double)x.b[0][1] - (double)x.b[0][0];
  const double sv = (double)x.b[1][1] - (double)x.b[1][0];
  const double sw = (double)x.b[2][1] - (double)x.b[2][0];
  if (sw <= su && sw <= sv) return 0;
  if (sv <= su && sv <= sw) return 1;
  if (su <= sv && su <= sw) return 2;
  return 0;
}
TMC_HD_COLD int plane_from_extent_f64(const Boxes& bx, int t) { return plane_from_extent(bx, t); }
TMC_HD_COLD int plane_from_gradient_exact(const float* pts, int n, Corners u) {
  const Point64 pd = mean_point_exact(pts, n);
  double f[8];
  for (int q = 0; q < 8; q++) f[q] = u.f[q];
  return plane_from_gradient(f, pd.p);
}

struct TailOut {
  float p[3];
  double p64[3];  // the representative in float64: the mean point itself when nothing is found
  int fail2;
};
TMC_HD_COLD TailOut representative_tail(Corners u, double iso, uint64_t c, int t, const float* pts, int n,
                                        const Boxes& bx, int prj);

// edge points of contour t (flat edge positions tstart .. tstart + n) recomputed from the corners
TMC_HD void contour_points(const float u[8], double iso, uint64_t c, int tstart, int n, float pts[36]) {
  const ff iso_ff = ffx::ff_from_double(iso);
  for (int q = 0; q < n; q++) {
    const int e = cedge(c, tstart + q);
    bool fb = false;
    const float l = edge_param_fast(e, u, iso, iso_ff, fb);
    local_from_param(e, l, pts + 3 * q);
  }
}
// float64 plane decision from the gradient at the reference's float64 mean point, with the points
// recomputed (rare: only when the float32 decision is within its error bound)
TMC_HD_COLD int plane_from_gradient_recomputed(Corners u, double iso, uint64_t c, int tstart, int n) {
  float pts[36];
  contour_points(u.f, iso, c, tstart, n, pts);
  return plane_from_gradient_exact(pts, n, u);
}

// Projection set-up of contour t from its coordinate sums s (float-float, in contour order) and its
// box: plane, permuted corners, mean point, sample coordinates and the w window.  Returns the
// plane; f64_coords counts sample coordinates computed in float64.  pts (the edge points) is only
// read by a rare float64 plane decision; without it (null) the points are recomputed from tstart.
TMC_HD int projection_setup_core(const float u[8], double iso, uint64_t c, int t, const ff s[3], int n,
                                 const float box[3][2], const float* pts, int tstart, ProjCtx& P, float us[7],
                                 float vs[7], int& f64_coords) {
  const int cnt_sz = csize(c, t);
  const ff nn = ffx::ff_from((float)n);
  const ff pm[3] = {ffx::ff_div(s[0], nn), ffx::ff_div(s[1], nn), ffx::ff_div(s[2], nn)};
  int prj;
  if (cnt_sz >= 6) {
    prj = plane_from_gradient_f(u, pm[0].hi, pm[1].hi, pm[2].hi);
    if (prj < 0) {
      Corners uc;
      for (int q = 0; q < 8; q++) uc.f[q] = u[q];
      prj = pts ? plane_from_gradient_exact(pts, n, uc) : plane_from_gradient_recomputed(uc, iso, c, tstart, n);
    }
  } else {
    prj = plane_from_extent_box_ff(box);
    if (prj < 0) {
      Box3 x;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        x.b[d][0] = box[d][0];
        x.b[d][1] = box[d][1];
      }
      prj = plane_from_extent_box_f64(x);
    }
  }
  uint32_t perm;
  plane(prj, P.A, P.B, P.W, perm);
#pragma unroll
  for (int q = 0; q < 8; q++) P.fp[q] = corner_at(u, (perm >> (4 * q)) & 0xF);
  P.sabs_lo = fmaxf(fmaxf(fabsf(P.fp[0]), fabsf(P.fp[1])), fmaxf(fabsf(P.fp[2]), fabsf(P.fp[3])));
  P.sabs_hi = fmaxf(fmaxf(fabsf(P.fp[4]), fabsf(P.fp[5])), fmaxf(fabsf(P.fp[6]), fabsf(P.fp[7])));
  P.pff[0] = P.A == 0 ? pm[0] : pm[1];
  P.pff[1] = P.B == 1 ? pm[1] : pm[2];
  P.pff[2] = P.W == 2 ? pm[2] : (P.W == 1 ? pm[1] : pm[0]);
  for (int d = 0; d < 3; d++) P.pf[d] = P.pff[d].hi;
  P.iso_ff = ffx::ff_from_double(iso);
  P.iso_d = iso;
  P.iso_f = (float)iso;
  P.iso_err = fabsf((float)(iso - (double)P.iso_f)) + fabsf(P.iso_f) * 0x1p-30f;
  P.cnt = ccount(c);
  P.excl = P.cnt != 1 && cnt_sz != 3;
  P.t = t;
  P.c = c;
  P.bx = nullptr;
  const float umin = P.A == 0 ? box[0][0] : box[1][0], umax = P.A == 0 ? box[0][1] : box[1][1];
  const float vmin = P.B == 1 ? box[1][0] : box[2][0], vmax = P.B == 1 ? box[1][1] : box[2][1];
  const float wlo = P.W == 2 ? box[2][0] : (P.W == 1 ? box[1][0] : box[0][0]);
  const float whi = P.W == 2 ? box[2][1] : (P.W == 1 ? box[1][1] : box[0][1]);
  sample_coords(umin, umax, us, f64_coords);
  sample_coords(vmin, vmax, vs, f64_coords);
  w_window(wlo, whi, P.wlo, P.whi);
  return prj;
}

// The same from the contour's edge points and the boxes of all the cell's contours (the boxes of
// the others serve the neighbour-contour exclusion of the sample evaluation).
TMC_HD int projection_setup(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                            const Boxes& bx, ProjCtx& P, float us[7], float vs[7], int& f64_coords) {
  ff s[3] = {ffx::ff_from(0.0f), ffx::ff_from(0.0f), ffx::ff_from(0.0f)};
#pragma unroll 1
  for (int q = 0; q < n; q++) {
    s[0] = ffx::ff_add(s[0], ffx::ff_from(pts[3 * q]));
    s[1] = ffx::ff_add(s[1], ffx::ff_from(pts[3 * q + 1]));
    s[2] = ffx::ff_add(s[2], ffx::ff_from(pts[3 * q + 2]));
  }
  const int prj = projection_setup_core(u, iso, c, t, s, n, bx.b[t], pts, 0, P, us, vs, f64_coords);
  P.bx = &bx;
  return prj;
}

// Contour t's coordinate sums and box accumulated while its edge points are computed (edge order,
// as projection_setup sums them), without keeping the points.
struct ContourAcc {
  ff s[3];
  float box[3][2];
};
TMC_HD void contour_acc(const float u[8], double iso, ff iso_ff, uint64_t c, int tstart, int n, ContourAcc& A) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    A.s[d] = ffx::ff_from(0.0f);
    A.box[d][0] = 1;
    A.box[d][1] = 0;
  }
#pragma unroll 1
  for (int q = 0; q < n; q++) {
    const int e = cedge(c, tstart + q);
    bool fb = false;
    const float l = edge_param_fast(e, u, iso, iso_ff, fb);
    float ui[3];
    local_from_param(e, l, ui);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      A.s[d] = ffx::ff_add(A.s[d], ffx::ff_from(ui[d]));
      A.box[d][0] = A.box[d][0] > ui[d] ? ui[d] : A.box[d][0];
      A.box[d][1] = A.box[d][1] < ui[d] ? ui[d] : A.box[d][1];
    }
  }
}

// 7x7 projection of contour t.  pts: the contour's edge points (3 floats each, in contour order),
// n of them.  Returns true with p_out (local coordinates) set when a valid sample exists; false
// when the reference goes on to its 26x26 retry (representative_tail, or the lane-split retry).
TMC_HD bool representative_7x7(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                               const Boxes& bx, float p_out[3], Stats& st, float* buf, int stride, int& prj) {
  ProjCtx P;
  float us[7], vs[7];
  int f64_samples = 0;
  prj = projection_setup(u, iso, c, t, pts, n, bx, P, us, vs, f64_samples);
  float pt[3];
  const int r = projection_fast<true>(P, us, vs, pt, buf, stride, f64_samples, pts, n);
  st.fallback += f64_samples;
  if (r != 0) return false;
  p_out[P.A] = pt[0];
  p_out[P.B] = pt[1];
  p_out[P.W] = pt[2];
  return true;
}

// Representative of contour t.  On return p_out holds the local coordinates (floats) of the
// representative and p64 the float64 value the reference places the vertex at: the same floats,
// except when no sample is valid even at 26x26 (the reference then keeps its float64 mean point,
// unrounded).
TMC_HD void representative_fast(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                                const Boxes& bx, float p_out[3], Stats& st, float* buf, int stride,
                                double p64[3]) {
  int prj = 0;
  if (representative_7x7(u, iso, c, t, pts, n, bx, p_out, st, buf, stride, prj)) {
    for (int d = 0; d < 3; d++) p64[d] = p_out[d];
    return;
  }
  // no valid 7x7 sample
  st.fail1++;
  Corners uc;
  for (int q = 0; q < 8; q++) uc.f[q] = u[q];
  const TailOut tail = representative_tail(uc, iso, c, t, pts, n, bx, prj);
  st.fail2 += tail.fail2;
  for (int d = 0; d < 3; d++) {
    p_out[d] = tail.p[d];
    p64[d] = tail.p64[d];
  }
}

// ---------------------------------------------------------------------------------------------
// two-pass form: a set-up pass writes one ProjRecord per vertex, a projection pass reads it.  Each
// pass is a small kernel (registers, instruction cache); contours that need anything beyond the
// float32 / float-float path (the neighbour-contour exclusion, a float64 sample, the 26x26 tail) are
// left to the one-pass kernel.
// ---------------------------------------------------------------------------------------------
struct alignas(16) ProjRecord {
  float fp[8];        // corner values permuted to the projection frame
  float us[7], vs[7];  // sample coordinates
  float wlo, whi;      // w window
  float pff[6];        // mean point in the projection frame, float pairs (hi, lo)
  double iso;
  int32_t prj;         // projection plane (0..2)
  int32_t pad;
  float iso_hi, iso_lo;  // iso as a float pair (ffx::ff_from_double), made once per volume
};

// Set-up pass of one contour.  Returns false when the contour needs the one-pass kernel.
TMC_HD bool projection_record(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                              const Boxes& bx, ProjRecord& R, int& f64_coords) {
  ProjCtx P;
  const int prj = projection_setup(u, iso, c, t, pts, n, bx, P, R.us, R.vs, f64_coords);
  if (P.excl) return false;
  for (int q = 0; q < 8; q++) R.fp[q] = P.fp[q];
  R.wlo = P.wlo;
  R.whi = P.whi;
  for (int d = 0; d < 3; d++) {
    R.pff[2 * d] = P.pff[d].hi;
    R.pff[2 * d + 1] = P.pff[d].lo;
  }
  R.iso = iso;
  R.prj = prj;
  R.pad = 0;
  R.iso_hi = P.iso_ff.hi;
  R.iso_lo = P.iso_ff.lo;
  return true;
}

// Set-up pass of contour t (edges tstart .. tstart + n of the cell's contour word c) from its
// accumulated sums and box; returns false when the contour needs the one-pass kernel.
TMC_HD bool projection_record_acc(const float u[8], double iso, uint64_t c, int t, int tstart, int n,
                                  const ContourAcc& A, ProjRecord& R, int& f64_coords) {
  if (ccount(c) != 1 && csize(c, t) != 3) return false;  // neighbour-contour exclusion applies
  ProjCtx P;
  const int prj = projection_setup_core(u, iso, c, t, A.s, n, A.box, nullptr, tstart, P, R.us, R.vs, f64_coords);
  for (int q = 0; q < 8; q++) R.fp[q] = P.fp[q];
  R.wlo = P.wlo;
  R.whi = P.whi;
  for (int d = 0; d < 3; d++) {
    R.pff[2 * d] = P.pff[d].hi;
    R.pff[2 * d + 1] = P.pff[d].lo;
  }
  R.iso = iso;
  R.prj = prj;
  R.pad = 0;
  R.iso_hi = P.iso_ff.hi;
  R.iso_lo = P.iso_ff.lo;
  return true;
}

// Projection pass: 0 = found (p set, local coordinates), 1 = no valid sample, 2 = a sample distance
// needs float64.  The last two go to the one-pass kernel.  f64 counts values recomputed in float64.
// projection state of a record (contours with a record have no neighbour-contour exclusion)
TMC_HD void ctx_from_record(const ProjRecord& R, ProjCtx& P) {
  uint32_t perm;
  plane(R.prj, P.A, P.B, P.W, perm);
#pragma unroll
  for (int q = 0; q < 8; q++) P.fp[q] = R.fp[q];
  P.sabs_lo = fmaxf(fmaxf(fabsf(P.fp[0]), fabsf(P.fp[1])), fmaxf(fabsf(P.fp[2]), fabsf(P.fp[3])));
  P.sabs_hi = fmaxf(fmaxf(fabsf(P.fp[4]), fabsf(P.fp[5])), fmaxf(fabsf(P.fp[6]), fabsf(P.fp[7])));
  for (int d = 0; d < 3; d++) {
    P.pff[d] = ff{R.pff[2 * d], R.pff[2 * d + 1]};
    P.pf[d] = R.pff[2 * d];
  }
  P.iso_ff = ff{R.iso_hi, R.iso_lo};  // no float64 conversion per vertex
  P.iso_d = R.iso;
  P.iso_f = P.iso_ff.hi;
  P.iso_err = fabsf(P.iso_ff.lo) + fabsf(P.iso_ff.hi) * 0x1p-30f;
  P.cnt = 1;
  P.excl = false;
  P.t = 0;
  P.c = 0;
  P.bx = nullptr;
  P.wlo = R.wlo;
  P.whi = R.whi;
}

TMC_HD int projection_from_record(const ProjRecord& R, float p_out[3], float* buf, int stride, int& f64) {
  ProjCtx P;
  ctx_from_record(R, P);
  float pt[3];
  const int r = projection_fast<false>(P, R.us, R.vs, pt, buf, stride, f64, nullptr, 0);
  if (r == 0) {
    p_out[P.A] = pt[0];
    p_out[P.B] = pt[1];
    p_out[P.W] = pt[2];
  }
  return r;
}

// ---------------------------------------------------------------------------------------------
// lane-split forms: the samples of one contour are spread over a group of lanes, lane l of nl
// evaluating samples l, l + nl, ... exactly (no pruning), and the lanes' winners are combined by
// (distance, loop index) -- the reference's strict `minDistance > d` over its loop order keeps the
// first of equal distances.  A 26x26 retry then costs ~22 samples per lane of a warp instead of 676
// on one thread, and a small mesh's 7x7 projections a few samples per lane.
// ---------------------------------------------------------------------------------------------
struct LaneBest {
  float d, w;
  int q;  // sample index i * ns + j in the reference's loop order; kNoSample when none is valid
};
constexpr int kNoSample = 0x7fffffff;
TMC_HD LaneBest lane_none() { return LaneBest{INFINITY, 0.0f, kNoSample}; }
TMC_HD bool lane_better(const LaneBest& a, const LaneBest& b) { return a.d < b.d || (a.d == b.d && a.q < b.q); }

// u_i = fl32(umin + i*(umax-umin)/27), i = 1..26: the 26x26 retry's coordinates, in float64 as the
// reference computes them (projection with nrSamples = 28, cpp_dmc/DualMarchingCubes.cpp:284-299)
TMC_HD float tail_coord(float lo, float hi, int i) {
  const double du = ((double)hi - (double)lo) / 27;
  return (float)((double)lo + i * du);
}

// The lane's share of the ns x ns samples at (us[i], vs[j]).  Samples whose float-float distance
// cannot be certified are evaluated in float64 from the mean point of pts.  f64 counts values
// computed in float64.
TMC_HD LaneBest grid_lane(const ProjCtx& P, const float* us, const float* vs, int ns, int lane, int nl,
                          const float* pts, int npts, int& f64) {
  LaneBest b = lane_none();
  bool have_pd = false;
  double pd[3] = {0, 0, 0};
#pragma unroll 1
  for (int q = lane; q < ns * ns; q += nl) {
    const int i = q / ns, j = q - i * ns;
    SampleOut s = sample_exact(P, us[i], vs[j]);
    f64 += s.f64;
    if (s.status == 2) {
      if (!have_pd) {
        const Point64 pm = mean_point_exact(pts, npts);
        pd[0] = pm.p[P.A];
        pd[1] = pm.p[P.B];
        pd[2] = pm.p[P.W];
        have_pd = true;
      }
      s = sample_f64(P, pd[0], pd[1], pd[2], us[i], vs[j]);
      f64++;
    }
    // the reference's minDistance starts at 100 (float64): a sample must be closer to count
    if (s.status != 1 || !(s.d < 100.0f)) continue;
    if (s.d < b.d) {  // the lane's samples come in loop order: the first of equal distances stays
      b.d = s.d;
      b.w = s.w;
      b.q = q;
    }
  }
  return b;
}

// The lane's share of a record's 7x7 samples, all evaluated exactly without float64 distances:
// `uncertain` is set when a distance cannot be certified, and the vertex then goes to the one-pass
// kernels like the single-thread pass's.
TMC_HD LaneBest record_lane(const ProjCtx& P, const ProjRecord& R, int lane, int nl, int& f64, bool& uncertain) {
  LaneBest b = lane_none();
#pragma unroll 1
  for (int q = lane; q < 49; q += nl) {
    const int i = q / 7, j = q - i * 7;
    const SampleOut s = sample_exact(P, R.us[i], R.vs[j]);
    f64 += s.f64;
    if (s.status == 2) uncertain = true;
    if (s.status != 1 || !(s.d < 100.0f)) continue;
    if (s.d < b.d) {
      b.d = s.d;
      b.w = s.w;
      b.q = q;
    }
  }
  return b;
}

// Local coordinates of the winning sample b of an ns x ns grid.
TMC_HD void lane_point(const ProjCtx& P, const float* us, const float* vs, int ns, const LaneBest& b, float p[3]) {
  const int i = b.q / ns, j = b.q - i * ns;
  p[P.A] = us[i];
  p[P.B] = vs[j];
  p[P.W] = b.w;
}

// Host forms (the lanes run one after another and are combined as the device combines them).
// The lane-split representative, 7x7 and retry alike; returns what representative_fast returns.
inline void representative_lanes_host(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                                      const Boxes& bx, float p_out[3], double p64[3], Stats& st) {
  ProjCtx P;
  float us[26], vs[26];
  int f64 = 0;
  projection_setup(u, iso, c, t, pts, n, bx, P, us, vs, f64);
  LaneBest b = lane_none();
  for (int lane = 0; lane < 32; lane++) {
    const LaneBest x = grid_lane(P, us, vs, 7, lane, 32, pts, n, f64);
    if (lane_better(x, b)) b = x;
  }
  int ns = 7;
  if (b.q == kNoSample) {
    st.fail1++;
    for (int a = 0; a < 26; a++) {
      us[a] = tail_coord(bx.b[t][P.A][0], bx.b[t][P.A][1], a + 1);
      vs[a] = tail_coord(bx.b[t][P.B][0], bx.b[t][P.B][1], a + 1);
    }
    ns = 26;
    for (int lane = 0; lane < 32; lane++) {
      const LaneBest x = grid_lane(P, us, vs, 26, lane, 32, pts, n, f64);
      if (lane_better(x, b)) b = x;
    }
  }
  st.fallback += f64;
  if (b.q != kNoSample) {
    lane_point(P, us, vs, ns, b, p_out);
    for (int d = 0; d < 3; d++) p64[d] = p_out[d];
    return;
  }
  st.fail2++;
  const Point64 pm = mean_point_exact(pts, n);
  for (int d = 0; d < 3; d++) {
    p64[d] = pm.p[d];
    p_out[d] = (float)pm.p[d];
  }
}
// The lane-group projection pass (nl lanes per record); returns 0 (p_out set), 1 (no valid sample)
// or 2 (a distance needs float64), as projection_from_record.
inline int projection_from_record_lanes_host(const ProjRecord& R, int nl, float p_out[3]) {
  ProjCtx P;
  ctx_from_record(R, P);
  LaneBest b = lane_none();
  bool unc = false;
  int f64 = 0;
  for (int lane = 0; lane < nl; lane++) {
    const LaneBest x = record_lane(P, R, lane, nl, f64, unc);
    if (lane_better(x, b)) b = x;
  }
  if (unc) return 2;
  if (b.q == kNoSample) return 1;
  lane_point(P, R.us, R.vs, 7, b, p_out);
  return 0;
}

// The 7x7 projection is empty: the reference then tries 26x26 samples from the mean point, in
// float64, and keeps the mean point when that finds nothing either.
TMC_HD_COLD TailOut representative_tail(Corners u, double iso, uint64_t c, int t, const float* pts, int n,
                                        const Boxes& bx, int prj) {
  const Point64 pm = mean_point_exact(pts, n);
  int A, B, W;
  uint32_t perm;
  plane(prj, A, B, W, perm);
  double fp[8];
  for (int q = 0; q < 8; q++) fp[q] = (double)u.f[(perm >> (4 * q)) & 0xF];
  double pd[3] = {pm.p[0], pm.p[1], pm.p[2]};
  double ptd[3] = {pd[A], pd[B], pd[W]};
  TailOut r;
  r.fail2 = projection_exact(fp, iso, c, t, ptd, bx, A, B, W, 28) ? 0 : 1;
  pd[A] = ptd[0];
  pd[B] = ptd[1];
  pd[W] = ptd[2];
  for (int d = 0; d < 3; d++) {
    r.p64[d] = pd[d];
    r.p[d] = (float)pd[d];
  }
  return r;
}

}  // namespace repr
}  // namespace tmc
