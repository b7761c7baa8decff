// CPU check of the DMC vertex representative: for every contour of a field, the fast path
// (float32 search + certified float-float rounding, tmc_gb300/csrc/dmc_repr.cuh) must return the
// same floats as the float64 restatement of the reference.  Built with nvcc as host code.
//   repr_check field.raw nx ny nz iso  -> prints "contours mismatches fallbacks fail1 fail2"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../tmc_gb300/csrc/common.cuh"
#include "../../tmc_gb300/csrc/dmc_repr.cuh"

using namespace tmc;

static long g_decider_mismatch = 0;
static uint64_t polygon(unsigned cs, const float u[8], double iso) {
  if (!case_ambiguous(cs)) return table_contour(TMC_CASE_CONTOUR[cs]);
  uint64_t to = ~0ull;
  for (int f = 0; f < 6; f++) {
    const uint32_t fv = face_v_pack(f);
    const int fc = face_case(cs, fv);
    int sep = 0;
    if (fc == 6 || fc == 9) {
      const float a = u[nib(fv, 0)], b = u[nib(fv, 1)], c = u[nib(fv, 2)], d = u[nib(fv, 3)];
      sep = decider(a, b, c, d) >= iso;
      // the float-float decision used on the GPU must agree
      if (decider_ge(a, b, c, d, iso, ffx::ff_from_double(iso)) != (bool)sep) g_decider_mismatch++;
    }
    face_segments(fc, sep, face_e_pack(f), to);
  }
  return connect_contours(to, case_edge_mask(cs));
}

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
  const double iso = atof(argv[5]);
  std::vector<float> f((size_t)nx * ny * nz);
  FILE* in = fopen(argv[1], "rb");
  if (!in || fread(f.data(), 4, f.size(), in) != f.size()) return 3;
  fclose(in);
  const float iso_up = [&] { float x = (float)iso; if ((double)x < iso) x = nextafterf(x, INFINITY); return x; }();
  long contours = 0, mism = 0, two_pass = 0;
  repr::Stats se, sf, sl;
  for (int k = 0; k < nz - 1; k++)
    for (int j = 0; j < ny - 1; j++)
      for (int i = 0; i < nx - 1; i++) {
        float u[8];
        for (int q = 0; q < 8; q++)
          u[q] = f[((size_t)(k + ((q >> 2) & 1)) * ny + (j + ((q >> 1) & 1))) * nx + i + (q & 1)];
        unsigned cs = 0;
        for (int q = 0; q < 8; q++) cs |= (unsigned)(u[q] >= iso_up) << q;
        if (cs == 0 || cs == 255) continue;
        const uint64_t c = polygon(cs, u, iso);
        const int n = cnt_count(c);
        repr::Boxes bx;
        float pts[4][36];
        int flat = 0;
        for (int t = 0; t < n; t++) {
          for (int d = 0; d < 3; d++) { bx.b[t][d][0] = 1; bx.b[t][d][1] = 0; }
          const int sz = cnt_size(c, t);
          for (int q = 0; q < sz; q++) {
            const int e = cnt_edge(c, flat + q);
            bool fb = false;
            const float l = repr::edge_param_fast(e, u, iso, ffx::ff_from_double(iso), fb);
            if (l != repr::edge_param_exact(e, u, iso)) mism++;
            float ui[3];
            repr::local_from_param(e, l, ui);
            for (int d = 0; d < 3; d++) {
              pts[t][3 * q + d] = ui[d];
              bx.b[t][d][0] = bx.b[t][d][0] > ui[d] ? ui[d] : bx.b[t][d][0];
              bx.b[t][d][1] = bx.b[t][d][1] < ui[d] ? ui[d] : bx.b[t][d][1];
            }
          }
          flat += sz;
        }
        for (int t = 0; t < n; t++) {
          const int sz = cnt_size(c, t);
          const repr::Point64 pm = repr::mean_point_exact(pts[t], sz);
          double pe[3] = {pm.p[0], pm.p[1], pm.p[2]};
          repr::representative_exact(u, iso, c, t, pe, bx, se);
          float pf[3];
          float lb[49];
          double p64[3];
          repr::representative_fast(u, iso, c, t, pts[t], sz, bx, pf, sf, lb, 1, p64);
          // the float64 position the reference uses (its mean point, unrounded, when nothing is found)
          if (pe[0] != p64[0] || pe[1] != p64[1] || pe[2] != p64[2]) {
            if (mism < 5) fprintf(stderr, "float64 representative differs cell %d %d %d t %d\n", i, j, k, t);
            mism++;
          }
          // the lane-split form (warp per vertex on the GPU) must agree everywhere
          {
            float pl[3];
            double pl64[3];
            repr::representative_lanes_host(u, iso, c, t, pts[t], sz, bx, pl, pl64, sl);
            if (pl[0] != pf[0] || pl[1] != pf[1] || pl[2] != pf[2] || pl64[0] != p64[0] || pl64[1] != p64[1] ||
                pl64[2] != p64[2]) {
              if (mism < 5) fprintf(stderr, "lane-split differs cell %d %d %d t %d\n", i, j, k, t);
              mism++;
            }
          }
          // the two-pass form must agree wherever it applies
          {
            repr::ProjRecord R;
            int f64c = 0;
            std::memset(&R, 0, sizeof R);  // the record's tail padding is compared too
            const bool rec_ok = repr::projection_record(u, iso, c, t, pts[t], sz, bx, R, f64c);
            {
              // the set-up kernel's form: sums and box accumulated without the point array
              int tstart = 0;
              for (int t2 = 0; t2 < t; t2++) tstart += cnt_size(c, t2);
              repr::ContourAcc A;
              repr::contour_acc(u, iso, ffx::ff_from_double(iso), c, tstart, sz, A);
              repr::ProjRecord R2;
              std::memset(&R2, 0, sizeof R2);
              int f64a = 0;
              const bool acc_ok = repr::projection_record_acc(u, iso, c, t, tstart, sz, A, R2, f64a);
              if (acc_ok != rec_ok || (rec_ok && (std::memcmp(&R, &R2, sizeof R) != 0 || f64a != f64c))) {
                if (mism < 5) fprintf(stderr, "accumulated set-up differs cell %d %d %d t %d\n", i, j, k, t);
                mism++;
              }
            }
            if (rec_ok) {
              float pr[3];
              int f64r = 0;
              const int rr = repr::projection_from_record(R, pr, lb, 1, f64r);
              // the lane-group form of the same pass (small meshes) must agree where it finds a point
              for (int nl : {4, 8, 32}) {
                float pg[3];
                const int rg = repr::projection_from_record_lanes_host(R, nl, pg);
                if (rg == 0 && (pg[0] != pf[0] || pg[1] != pf[1] || pg[2] != pf[2] || rr == 1)) {
                  if (mism < 5) fprintf(stderr, "lane-group projection differs cell %d %d %d t %d\n", i, j, k, t);
                  mism++;
                }
                if (rg == 1 && rr == 0) mism++;  // a certain empty projection cannot have a winner
              }
              if (rr == 0) {
                two_pass++;
                if (pr[0] != pf[0] || pr[1] != pf[1] || pr[2] != pf[2]) {
                  if (mism < 5) fprintf(stderr, "two-pass differs cell %d %d %d t %d\n", i, j, k, t);
                  mism++;
                }
              }
            }
          }
          contours++;
          if ((float)pe[0] != pf[0] || (float)pe[1] != pf[1] || (float)pe[2] != pf[2]) {
            if (mism < 5)
              fprintf(stderr, "cell %d %d %d t %d: exact %.9g %.9g %.9g fast %.9g %.9g %.9g\n", i, j, k, t, pe[0],
                      pe[1], pe[2], pf[0], pf[1], pf[2]);
            mism++;
          }
        }
      }
  mism += g_decider_mismatch;
  if (sl.fail1 != se.fail1 || sl.fail2 != se.fail2) {
    fprintf(stderr, "lane-split failure counters %d %d\n", sl.fail1, sl.fail2);
    mism++;
  }
  printf("%ld %ld %d %d %d %d %d %ld\n", contours, mism, sf.fallback, sf.fail1, sf.fail2, se.fail1, se.fail2, two_pass);
  return 0;
}
