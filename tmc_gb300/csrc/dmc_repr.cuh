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
};

// ---------------------------------------------------------------------------------------------
// edge parameter: getLocalCoordinates (cpp_dmc/DualMarchingCubes.h:391-407), l rounded to float
// ---------------------------------------------------------------------------------------------
TMC_HD_COLD float edge_param_exact(int e, const float u[8], double iso) {
  const int v0 = nibr(EDGE_V0, e), v1 = nibr(EDGE_V1, e);
  return (float)((iso - (double)u[v0]) / ((double)u[v1] - (double)u[v0]));
}

TMC_HD float edge_param_fast(int e, const float u[8], double iso, ff iso_ff, bool& fallback) {
  const int v0 = nibr(EDGE_V0, e), v1 = nibr(EDGE_V1, e);
  const float f0 = u[v0], f1 = u[v1];
  const ff num = ffx::ff_sub(iso_ff, ffx::ff_from(f0));
  const ff den = ffx::two_sum(f1, -f0);  // exact
  const ff q = ffx::ff_div(num, den);
  const float aq = fabsf(q.hi);
  const float mag = fmaxf(fabsf(iso_ff.hi), fabsf(f0));
  const float err = aq * 0x1p-42f + mag * 0x1p-45f / fabsf(den.hi);
  float l;
  if (ffx::ff_round(q, err, l)) return l;
  fallback = true;
  return edge_param_exact(e, u, iso);
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
struct SampleApprox {
  float D, ED;
  int status;  // 0 invalid, 1 valid, 2 uncertain
};

struct ProjCtx {
  float fp[8];          // permuted corner values
  float umin, vmin;     // sample grid origin
  float us[7], vs[7];   // exact sample coordinates
  float wlo, whi;       // w >= wlo && w <= whi  <=>  wmin <= w <= wmax (double bounds)
  float pf[3];          // mean point (approximate, |error| <= 2^-23)
  ff pff[3];            // mean point (float-float, within 2^-43 of the reference's double)
  float iso_f;
  float iso_err;        // |iso - iso_f|
  ff iso_ff;
  double iso_d;
  double pd[3];         // mean point in float64, permuted (valid when have_pd)
  bool have_pd;
  const float* pts;     // contour edge points (for the float64 mean)
  int npts;
  int f64_samples;      // samples evaluated in float64
  int cnt, cnt_sz, t, A, B, W;
  uint64_t c;
  const Boxes* bx;
};

// float32 evaluation of one sample with error bounds
TMC_HD SampleApprox sample_approx(const ProjCtx& P, float u, float v) {
  SampleApprox r;
  const float omu = 1 - u, omv = 1 - v;
  const float* f = P.fp;
  const float A1 = ffx::fma_rn(u, f[1], omu * f[0]), B1 = ffx::fma_rn(u, f[3], omu * f[2]);
  const float A2 = ffx::fma_rn(u, f[5], omu * f[4]), B2 = ffx::fma_rn(u, f[7], omu * f[6]);
  const float g1 = ffx::fma_rn(v, B1, omv * A1), g2 = ffx::fma_rn(v, B2, omv * A2);
  const float S1 = fabsf(omv) * (fabsf(omu * f[0]) + fabsf(u * f[1])) + fabsf(v) * (fabsf(omu * f[2]) + fabsf(u * f[3]));
  const float S2 = fabsf(omv) * (fabsf(omu * f[4]) + fabsf(u * f[5])) + fabsf(v) * (fabsf(omu * f[6]) + fabsf(u * f[7]));
  const float Eg1 = S1 * 0x1p-20f + fabsf(g1) * 0x1p-23f;
  const float Eg2 = S2 * 0x1p-20f + fabsf(g2) * 0x1p-23f;
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
  if (status != 0 && P.cnt != 1 && P.cnt_sz != 3) {
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

// One exactly evaluated sample.  Results are returned by value: the out-of-line evaluators write
// nothing through pointers into the caller's frame.
struct SampleOut {
  float w, d;
  int status;  // 0 invalid, 1 valid, 2 rounding not certified (evaluate in float64)
};

// float64 evaluation of one sample, as the reference's loop body (projection, :298-316)
TMC_HD_COLD SampleOut sample_f64(const ProjCtx& P, double pd0, double pd1, double pd2, float u, float v) {
  SampleOut r{0.0f, 0.0f, 0};
  double fp[8];
  for (int q = 0; q < 8; q++) fp[q] = P.fp[q];
  const float g1 = (1 - v) * ((1 - u) * fp[0] + u * fp[1]) + v * ((1 - u) * fp[2] + u * fp[3]);
  const float g2 = (1 - v) * ((1 - u) * fp[4] + u * fp[5]) + v * ((1 - u) * fp[6] + u * fp[7]);
  if (g1 == g2) return r;
  const float w = (P.iso_d - g1) / (g2 - g1);
  if (!(w >= P.wlo && w <= P.whi)) return r;
  if (P.cnt != 1 && P.cnt_sz != 3 && in_neighbor_bbox(u, v, w, P.c, P.t, *P.bx, P.A, P.B, P.W)) return r;
  r.status = 1;
  r.w = w;
  r.d = (pd0 - u) * (pd0 - u) + (pd1 - v) * (pd1 - v) + (pd2 - w) * (pd2 - w);
  return r;
}

// exact evaluation of one sample (status 2 when a rounding cannot be certified)
TMC_HD_COLD SampleOut sample_exact(const ProjCtx& P, float u, float v) {
  SampleOut r{0.0f, 0.0f, 2};
  const float omu = 1 - u, omv = 1 - v;
  const float* f = P.fp;
  const ff A1 = ffx::ff_add(ffx::two_prod(omu, f[0]), ffx::two_prod(u, f[1]));
  const ff B1 = ffx::ff_add(ffx::two_prod(omu, f[2]), ffx::two_prod(u, f[3]));
  const ff A2 = ffx::ff_add(ffx::two_prod(omu, f[4]), ffx::two_prod(u, f[5]));
  const ff B2 = ffx::ff_add(ffx::two_prod(omu, f[6]), ffx::two_prod(u, f[7]));
  const ff G1 = ffx::ff_add(ffx::ff_mul_f(A1, omv), ffx::ff_mul_f(B1, v));
  const ff G2 = ffx::ff_add(ffx::ff_mul_f(A2, omv), ffx::ff_mul_f(B2, v));
  const float S1 = fabsf(omv) * (fabsf(omu * f[0]) + fabsf(u * f[1])) + fabsf(v) * (fabsf(omu * f[2]) + fabsf(u * f[3]));
  const float S2 = fabsf(omv) * (fabsf(omu * f[4]) + fabsf(u * f[5])) + fabsf(v) * (fabsf(omu * f[6]) + fabsf(u * f[7]));
  float g1, g2;
  if (!ffx::ff_round(G1, S1 * 0x1p-45f, g1)) return r;
  if (!ffx::ff_round(G2, S2 * 0x1p-45f, g2)) return r;
  if (g1 == g2) {
    r.status = 0;
    return r;
  }
  const float den = g2 - g1;  // the reference subtracts the two floats
  const ff num = ffx::ff_sub(P.iso_ff, ffx::ff_from(g1));
  const ff W = ffx::ff_div(num, ffx::ff_from(den));
  const float errW = fabsf(W.hi) * 0x1p-42f + (fabsf(P.iso_ff.hi) * 0x1p-46f + fabsf(num.hi) * 0x1p-50f) / fabsf(den);
  float w;
  if (!ffx::ff_round(W, errW, w)) return r;
  bool valid = (w >= P.wlo && w <= P.whi);
  if (valid && P.cnt != 1 && P.cnt_sz != 3) {
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

// 0 = found (pt set), 1 = no valid sample.  buf: 49 slots (lower bound of each sample's distance,
// +inf for a certainly invalid sample), slot q at buf[q * stride] (shared memory on the GPU, one
// column per thread), so that every sample is approximated once.
TMC_HD int projection_fast(ProjCtx& P, float pt[3], float* buf, int stride) {
  const Boxes& bx = *P.bx;
  const float umin = bx.b[P.t][P.A][0], umax = bx.b[P.t][P.A][1];
  const float vmin = bx.b[P.t][P.B][0], vmax = bx.b[P.t][P.B][1];
  sample_coords(umin, umax, P.us, P.f64_samples);
  sample_coords(vmin, vmax, P.vs, P.f64_samples);
  // w window in float64, as the reference widens it (wmin -= 1e-5 when the box is flat)
  double wmin = bx.b[P.t][P.W][0], wmax = bx.b[P.t][P.W][1];
  if (fabs(wmax - wmin) < 1e-5) {
    wmin -= 1e-5;
    wmax += 1e-5;
  }
  P.wlo = ffx::f_ceil(wmin);
  P.whi = ffx::f_floor(wmax);
  // pass 1: every sample once; the smallest certain upper bound of a valid sample's distance
  // (loops kept rolled: 49 inlined copies of the sample code overflow the instruction cache)
  float m = INFINITY;
#pragma unroll 1
  for (int i = 0; i < 7; i++)
#pragma unroll 1
    for (int j = 0; j < 7; j++) {
      const SampleApprox s = sample_approx(P, P.us[i], P.vs[j]);
      if (s.status == 1) m = fminf(m, s.D + s.ED);
      buf[(7 * i + j) * stride] = (s.status == 0) ? INFINITY : s.D - s.ED;
    }
  // pass 2: exact evaluation of every sample that can still win, in the reference's loop order
  float best = 100.0f;
  bool found = false;
#pragma unroll 1
  for (int i = 0; i < 7; i++)
#pragma unroll 1
    for (int j = 0; j < 7; j++) {
      if (!(buf[(7 * i + j) * stride] <= m)) continue;
      SampleOut s = sample_exact(P, P.us[i], P.vs[j]);
      if (s.status == 2) {
        if (!P.have_pd) {
          const Point64 pm = mean_point_exact(P.pts, P.npts);
          P.pd[0] = pm.p[P.A];
          P.pd[1] = pm.p[P.B];
          P.pd[2] = pm.p[P.W];
          P.have_pd = true;
        }
        s = sample_f64(P, P.pd[0], P.pd[1], P.pd[2], P.us[i], P.vs[j]);
        P.f64_samples++;
      }
      if (s.status != 1) continue;
      if (best > s.d) {
        best = s.d;
        pt[0] = P.us[i];
        pt[1] = P.vs[j];
        pt[2] = s.w;
        found = true;
      }
    }
  return found ? 0 : 1;
}

struct TailOut {
  float p[3];
  int fail2;
};
TMC_HD_COLD TailOut representative_tail(const float* u, double iso, uint64_t c, int t, const float* pts, int n,
                                        const Boxes& bx, int prj);

// Representative of contour t.  pts: the contour's edge points (3 floats each, in contour order),
// n of them.  On return p holds the local coordinates (floats) of the representative.
TMC_HD void representative_fast(const float u[8], double iso, uint64_t c, int t, const float* pts, int n,
                                const Boxes& bx, float p_out[3], Stats& st, float* buf, int stride) {
  const int cnt_sz = csize(c, t);
  int prj;
  if (cnt_sz >= 6) {
    // gradient plane: decided in float64 (large contours are a small minority)
    const Point64 pd = mean_point_exact(pts, n);
    double f[8];
    for (int q = 0; q < 8; q++) f[q] = u[q];
    prj = plane_from_gradient(f, pd.p);
  } else {
    prj = plane_from_extent(bx, t);  // three float64 differences
  }
  ProjCtx P;
  uint32_t perm;
  plane(prj, P.A, P.B, P.W, perm);
  for (int q = 0; q < 8; q++) P.fp[q] = u[(perm >> (4 * q)) & 0xF];
  // mean point, float-float
  ff s[3] = {ffx::ff_from(0.0f), ffx::ff_from(0.0f), ffx::ff_from(0.0f)};
  for (int q = 0; q < n; q++)
    for (int d = 0; d < 3; d++) s[d] = ffx::ff_add(s[d], ffx::ff_from(pts[3 * q + d]));
  ff pm[3];
  for (int d = 0; d < 3; d++) pm[d] = ffx::ff_div(s[d], ffx::ff_from((float)n));
  P.pff[0] = pm[P.A];
  P.pff[1] = pm[P.B];
  P.pff[2] = pm[P.W];
  for (int d = 0; d < 3; d++) P.pf[d] = P.pff[d].hi;
  P.iso_ff = ffx::ff_from_double(iso);
  P.iso_d = iso;
  P.have_pd = false;
  P.pts = pts;
  P.npts = n;
  P.f64_samples = 0;
  P.iso_f = (float)iso;
  P.iso_err = fabsf((float)(iso - (double)P.iso_f)) + fabsf(P.iso_f) * 0x1p-30f;
  P.cnt = ccount(c);
  P.cnt_sz = cnt_sz;
  P.t = t;
  P.c = c;
  P.bx = &bx;
  float pt[3];
  const int r = projection_fast(P, pt, buf, stride);
  st.fallback += P.f64_samples;
  if (r == 0) {
    p_out[P.A] = pt[0];
    p_out[P.B] = pt[1];
    p_out[P.W] = pt[2];
    return;
  }
  // no valid 7x7 sample (r == 1)
  st.fail1++;
  const TailOut tail = representative_tail(u, iso, c, t, pts, n, bx, prj);
  st.fail2 += tail.fail2;
  p_out[0] = tail.p[0];
  p_out[1] = tail.p[1];
  p_out[2] = tail.p[2];
}

// The 7x7 projection is empty: the reference then tries 26x26 samples from the mean point, in
// float64, and keeps the mean point when that finds nothing either.
TMC_HD_COLD TailOut representative_tail(const float* u, double iso, uint64_t c, int t, const float* pts, int n,
                                        const Boxes& bx, int prj) {
  const Point64 pm = mean_point_exact(pts, n);
  int A, B, W;
  uint32_t perm;
  plane(prj, A, B, W, perm);
  double fp[8];
  for (int q = 0; q < 8; q++) fp[q] = (double)u[(perm >> (4 * q)) & 0xF];
  double pd[3] = {pm.p[0], pm.p[1], pm.p[2]};
  double ptd[3] = {pd[A], pd[B], pd[W]};
  TailOut r;
  r.fail2 = projection_exact(fp, iso, c, t, ptd, bx, A, B, W, 28) ? 0 : 1;
  pd[A] = ptd[0];
  pd[B] = ptd[1];
  pd[W] = ptd[2];
  r.p[0] = (float)pd[0];
  r.p[1] = (float)pd[1];
  r.p[2] = (float)pd[2];
  return r;
}

}  // namespace repr
}  // namespace tmc
