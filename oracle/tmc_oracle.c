/* CPU oracle for topologically correct Marching Cubes -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU path tmc::MarchingCubes::t_mc
 * (mc/MarchingCubes.cpp:151-317) with p_slice for the ambiguous cases (:323-1299): edge
 * vertices shared through a map keyed by 6*global_index + axis, table triangles (winding
 * reversed) for unambiguous cases, and for ambiguous cases the asymptotic decider with the
 * singular-face rule, the inner-ambiguity quadratic, the tunnel / inner hexagon and the
 * saddle inner vertex.  All in double precision, as the reference.
 *
 * key_bits = 32 reproduces the reference's int keys (which collide beyond ~2^31/6 grid points);
 * key_bits = 64 keys by the exact 64-bit global edge id.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load this library.
 */
#include <math.h>
#include <stdio.h>

#include "oracle_common.h"

/* ---------------------------------------------------------------------------------------- */
/* open-addressing map: edge key -> vertex index (std::map<int,int> m_vertices)              */
/* ---------------------------------------------------------------------------------------- */
typedef struct { int64_t* keys; int* vals; size_t cap, n; } kmap;
static uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}
static void kmap_init(kmap* m, size_t cap) {
  m->cap = 1; while (m->cap < cap) m->cap <<= 1;
  m->keys = (int64_t*)malloc(m->cap * sizeof(int64_t));
  m->vals = (int*)malloc(m->cap * sizeof(int));
  for (size_t i = 0; i < m->cap; i++) m->keys[i] = INT64_MIN;
  m->n = 0;
}
static void kmap_grow(kmap* m);
static int* kmap_slot(kmap* m, int64_t key, int* found) {
  if (2 * (m->n + 1) > m->cap) kmap_grow(m);
  size_t h = mix64((uint64_t)key) & (m->cap - 1);
  while (m->keys[h] != INT64_MIN && m->keys[h] != key) h = (h + 1) & (m->cap - 1);
  *found = m->keys[h] == key;
  if (!*found) { m->keys[h] = key; m->n++; }
  return &m->vals[h];
}
static void kmap_grow(kmap* m) {
  kmap o = *m;
  kmap_init(m, o.cap * 2);
  for (size_t i = 0; i < o.cap; i++)
    if (o.keys[i] != INT64_MIN) { int f; *kmap_slot(m, o.keys[i], &f) = o.vals[i]; }
  free(o.keys); free(o.vals);
}

typedef struct {
  const og_grid* g;
  const double* grad; /* 3 per grid point */
  double i0;
  int key_bits;
  kmap map;
  og_dvec pts, nrm;
  og_ivec tris;
  int64_t cases[11]; /* 3,4,5,6,6a,7,8,9,tunnel,12cont, singular errors */
} tmc_state;

/* UGrid::gradient (mc/MarchingCubes.cpp:1451-1509): one-sided differences on the border */
static double* tmc_gradient(const og_grid* g) {
  const size_t nr = (size_t)g->nx * g->ny * g->nz;
  double* gr = (double*)malloc(3 * nr * sizeof(double));
  const double dx = g->spacing[0], dy = g->spacing[1], dz = g->spacing[2];
  for (int k = 0; k < g->nz; k++)
    for (int j = 0; j < g->ny; j++)
      for (int i = 0; i < g->nx; i++) {
        double fx, fy, fz;
        if (i == 0) fx = (og_s(g, i + 1, j, k) - og_s(g, i, j, k)) / dx;
        else if (i == g->nx - 1) fx = (og_s(g, i, j, k) - og_s(g, i - 1, j, k)) / dx;
        else fx = (og_s(g, i + 1, j, k) - og_s(g, i - 1, j, k)) / (2 * dx);
        if (j == 0) fy = (og_s(g, i, j + 1, k) - og_s(g, i, j, k)) / dy;
        else if (j == g->ny - 1) fy = (og_s(g, i, j, k) - og_s(g, i, j - 1, k)) / dy;
        else fy = (og_s(g, i, j + 1, k) - og_s(g, i, j - 1, k)) / (2 * dy);
        if (k == 0) fz = (og_s(g, i, j, k + 1) - og_s(g, i, j, k)) / dz;
        else if (k == g->nz - 1) fz = (og_s(g, i, j, k) - og_s(g, i, j, k - 1)) / dz;
        else fz = (og_s(g, i, j, k + 1) - og_s(g, i, j, k - 1)) / (2 * dz);
        const size_t s = ((size_t)k * g->ny + j) * g->nx + i;
        gr[3 * s] = fx; gr[3 * s + 1] = fy; gr[3 * s + 2] = fz;
      }
  return gr;
}

static int64_t edge_key(tmc_state* st, int i, int j, int k, int e) {
  const og_grid* g = st->g;
  const int ix = i + OG_EDGE_GLOBAL[e][0], iy = j + OG_EDGE_GLOBAL[e][1], iz = k + OG_EDGE_GLOBAL[e][2];
  const int off = OG_EDGE_GLOBAL[e][3];
  if (st->key_bits == 32) {
    const unsigned gi = (unsigned)og_gindex(g, ix, iy, iz);
    return (int64_t)(int)(6u * gi + (unsigned)off);
  }
  const int64_t gl = (int64_t)iz * g->ny * g->nx + (int64_t)iy * g->nx + ix;
  return 6 * gl + off;
}

/* create or look up the vertex on edge e: interpolation as in t_mc (mc/MarchingCubes.cpp:241-268) */
static int edge_vertex(tmc_state* st, int i, int j, int k, int e, const double* u, double p[8][3], double n[8][3],
                       double* l_out) {
  const int v0 = OG_EDGE_V[e][0], v1 = OG_EDGE_V[e][1];
  const double l = (st->i0 - u[v0]) / (u[v1] - u[v0]);
  if (l_out) *l_out = l;
  double ip[3], in[3];
  for (int d = 0; d < 3; d++) ip[d] = (1 - l) * p[v0][d] + l * p[v1][d];
  for (int d = 0; d < 3; d++) in[d] = (1 - l) * n[v0][d] + l * n[v1][d];
  const double nl = sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
  in[0] = in[0] / nl; in[1] = in[1] / nl; in[2] = in[2] / nl;
  int found;
  int* slot = kmap_slot(&st->map, edge_key(st, i, j, k, e), &found);
  if (!found) {
    *slot = (int)(st->pts.n / 3);
    for (int d = 0; d < 3; d++) { og_dvec_push(&st->pts, ip[d]); og_dvec_push(&st->nrm, in[d]); }
  }
  return *slot;
}

static void push_tri(tmc_state* st, int a, int b, int c) {
  og_ivec_push(&st->tris, a); og_ivec_push(&st->tris, b); og_ivec_push(&st->tris, c);
}

/* trilinear interpolation inside the cell (the formula used for the inner vertices,
 * mc/MarchingCubes.cpp:950-955, :1213-1218) */
static void cell_trilinear(double q[8][3], double u, double v, double w, double out[3]) {
  for (int d = 0; d < 3; d++)
    out[d] = (1 - w) * ((1 - v) * (q[0][d] + u * (q[1][d] - q[0][d])) + v * (q[2][d] + u * (q[3][d] - q[2][d]))) +
             w * ((1 - v) * (q[4][d] + u * (q[5][d] - q[4][d])) + v * (q[6][d] + u * (q[7][d] - q[6][d])));
}

/* e_vert: local coordinate i of the point on edge e (mc/MarchingCubes.cpp:902-911) */
static const int EVERT[12][3] = {{3, 0, 0}, {1, 3, 0}, {3, 1, 0}, {0, 3, 0}, {3, 0, 1}, {1, 3, 1},
                                 {3, 1, 1}, {0, 3, 1}, {0, 0, 3}, {1, 0, 3}, {1, 1, 3}, {0, 1, 3}};
static double e_vert(const double* ecoord, int e, int i) {
  const int flag = EVERT[e][i];
  return flag == 3 ? ecoord[e] : (double)flag;
}

/* p_slice (mc/MarchingCubes.cpp:323-1299) */
static void p_slice(tmc_state* st, int i, int j, int k, const double* F, double p[8][3], double n[8][3], unsigned ic) {
  const double i0 = st->i0;
  int vidx[12];
  double ecoord[12];
  for (int e = 0; e < 12; e++) { vidx[e] = -1; ecoord[e] = 0; }
  for (int e = 0; e < 12; e++)
    if (TMC_EDGE_MASK[ic] & (1u << e)) vidx[e] = edge_vertex(st, i, j, k, e, F, p, n, &ecoord[e]);

  /* oriented segments with the decider (> / < / singular) (:495-668) */
  int to[12], f_flag[6] = {0, 0, 0, 0, 0, 0};
  for (int e = 0; e < 12; e++) to[e] = -1;
  for (int f = 0; f < 6; f++) {
    const int* fv = OG_FACE_V[f];
    const int* fe = OG_FACE_E[f];
    const double f0 = F[fv[0]], f1 = F[fv[1]], f2 = F[fv[2]], f3 = F[fv[3]];
    int fc = 0;
    if (f0 >= i0) fc |= 1;
    if (f1 >= i0) fc |= 2;
    if (f2 >= i0) fc |= 4;
    if (f3 >= i0) fc |= 8;
    int sep = 0;
    if (fc == 6 || fc == 9) {
      const double val = og_decider(f0, f1, f2, f3);
      if (val > i0) sep = 1;
      else if (val < i0) sep = 0;
      else {
        f_flag[f] = 1;
        /* singular face: decide by the edge parameters (e_flag = 0x218) */
        const unsigned short e_flag = 0x218;
        double ec0 = ecoord[fe[0]], ec1 = ecoord[fe[1]], ec2 = ecoord[fe[2]], ec3 = ecoord[fe[3]];
        if ((e_flag >> (f * 2)) & 1) { ec0 = 1 - ec0; ec2 = 1 - ec2; }
        if ((e_flag >> (f * 2)) & 2) { ec1 = 1 - ec1; ec3 = 1 - ec3; }
        const int cond1 = (ec1 < ec3 && ec0 > ec2), cond2 = (ec1 > ec3 && ec0 < ec2);
        if (!cond1 && !cond2) { st->cases[10]++; return; } /* "can't correctly triangulate" */
        if (fc == 6) sep = cond1 ? 0 : 1;
        else sep = cond1 ? 1 : 0;
      }
    }
    og_face_rule(fc, sep, fe, to);
  }
  og_contours c;
  og_connect(to, &c);

  /* intersection of the asymptotes: the inner-ambiguity quadratic (:715-795) */
  double ui[2] = {0, 0}, vi[2] = {0, 0}, wi[2] = {0, 0};
  unsigned q_sol = 0;
  const double a = (F[0] - F[1]) * (-F[6] + F[7] + F[4] - F[5]) - (F[4] - F[5]) * (-F[2] + F[3] + F[0] - F[1]);
  const double b = (i0 - F[0]) * (-F[6] + F[7] + F[4] - F[5]) + (F[0] - F[1]) * (F[6] - F[4]) -
                   (i0 - F[4]) * (-F[2] + F[3] + F[0] - F[1]) - (F[4] - F[5]) * (F[2] - F[0]);
  const double cc = (i0 - F[0]) * (F[6] - F[4]) - (i0 - F[4]) * (F[2] - F[0]);
  double d = b * b - 4 * a * cc;
  if (d > 0) {
    d = sqrt(d);
    ui[0] = (-b - d) / (2 * a);
    ui[1] = (-b + d) / (2 * a);
    double g1 = F[0] * (1 - ui[0]) + F[1] * ui[0];
    double g2 = F[2] * (1 - ui[0]) + F[3] * ui[0];
    vi[0] = (i0 - g1) / (g2 - g1);
    if (isnan(vi[0]) || isinf(vi[0])) vi[0] = -1.f;
    g1 = F[0] * (1 - ui[1]) + F[1] * ui[1];
    g2 = F[2] * (1 - ui[1]) + F[3] * ui[1];
    vi[1] = (i0 - g1) / (g2 - g1);
    if (isnan(vi[1]) || isinf(vi[1])) vi[1] = -1.f;
    g1 = F[0] * (1 - ui[0]) + F[1] * ui[0];
    g2 = F[4] * (1 - ui[0]) + F[5] * ui[0];
    wi[0] = (i0 - g1) / (g2 - g1);
    if (isnan(wi[0]) || isinf(wi[0])) wi[0] = -1.f;
    g1 = F[0] * (1 - ui[1]) + F[1] * ui[1];
    g2 = F[4] * (1 - ui[1]) + F[5] * ui[1];
    wi[1] = (i0 - g1) / (g2 - g1);
    if (isnan(wi[1]) || isinf(wi[1])) wi[1] = -1.f;
    if (f_flag[0]) { if (wi[0] < wi[1]) wi[0] = 0; else wi[1] = 0; }
    if (f_flag[1]) { if (wi[0] > wi[1]) wi[1] = 1; else wi[1] = 1; }
    if (f_flag[2]) { if (vi[0] < vi[1]) vi[0] = 0; else vi[1] = 0; }
    if (f_flag[3]) { if (vi[0] > vi[1]) vi[0] = 1; else vi[1] = 1; }
    if (f_flag[4]) { if (ui[0] < ui[1]) ui[0] = 0; else ui[1] = 0; }
    if (f_flag[5]) { if (ui[0] > ui[1]) ui[0] = 1; else ui[1] = 1; }
    if (0 < ui[0] && ui[0] < 1) q_sol |= 1;
    if (0 < ui[1] && ui[1] < 1) q_sol |= 2;
    if (0 < vi[0] && vi[0] < 1) q_sol |= 4;
    if (0 < vi[1] && vi[1] < 1) q_sol |= 8;
    if (0 < wi[0] && wi[0] < 1) q_sol |= 16;
    if (0 < wi[1] && wi[1] < 1) q_sol |= 32;
  }

  const int nbits = __builtin_popcount(q_sol);
  if (nbits == 6) {
    /* tunnel or a 12-vertex contour: inner hexagon (:831-1083) */
    st->cases[8]++;
    double hvt[6][3] = {{ui[0], vi[0], wi[0]}, {ui[0], vi[0], wi[1]}, {ui[1], vi[0], wi[1]},
                        {ui[1], vi[1], wi[1]}, {ui[1], vi[1], wi[0]}, {ui[0], vi[1], wi[0]}};
    int not_tunnel = 0xF;
    if (c.n == 3) {
      const double uc_min = (ui[0] < ui[1]) ? ui[0] : ui[1];
      const double uc_max = (ui[0] < ui[1]) ? ui[1] : ui[0];
      for (int t = 0; t < c.n; t++) {
        if (c.size[t] == 3) {
          double umin = 2, umax = -2;
          const int e0 = c.e[t][0], e1 = c.e[t][1], e2 = c.e[t][2];
          const double u_e0 = e_vert(ecoord, e0, 0), u_e1 = e_vert(ecoord, e1, 0), u_e2 = e_vert(ecoord, e2, 0);
          umin = (u_e0 < umin) ? u_e0 : umin;
          umin = (u_e1 < umin) ? u_e1 : umin;
          umin = (u_e2 < umin) ? u_e2 : umin;
          umax = (u_e0 > umax) ? u_e0 : umax;
          umax = (u_e1 > umax) ? u_e1 : umax;
          umax = (u_e2 > umax) ? u_e1 : umax; /* the reference compares u_e2 but keeps u_e1 */
          if (uc_min > umax || uc_max < umin) {
            not_tunnel = t;
            push_tri(st, vidx[e0], vidx[e1], vidx[e2]);
            st->cases[0]++;
          }
        }
      }
    }
    int tg[6];
    for (int s = 0; s < 6; s++) {
      double hp[3], hn[3];
      cell_trilinear(p, hvt[s][0], hvt[s][1], hvt[s][2], hp);
      cell_trilinear(n, hvt[s][0], hvt[s][1], hvt[s][2], hn);
      const double factor = sqrt(hn[0] * hn[0] + hn[1] * hn[1] + hn[2] * hn[2]);
      hn[0] = hn[0] / factor; hn[1] = hn[1] / factor; hn[2] = hn[2] / factor;
      tg[s] = (int)(st->pts.n / 3);
      for (int dd = 0; dd < 3; dd++) { og_dvec_push(&st->pts, hp[dd]); og_dvec_push(&st->nrm, hn[dd]); }
    }
    unsigned char tcon[12];
    for (int t = 0; t < c.n; t++) {
      if (not_tunnel == t) continue;
      const int sz = c.size[t];
      for (int r = 0; r < sz; r++) {
        unsigned idx = (unsigned)-1;
        double dist = 1000.;
        const int ci = c.e[t][r];
        const double ue = e_vert(ecoord, ci, 0), ve = e_vert(ecoord, ci, 1), we = e_vert(ecoord, ci, 2);
        for (int s = 0; s < 6; s++) {
          const double uval = ue - hvt[s][0], vval = ve - hvt[s][1], wval = we - hvt[s][2];
          const double val = uval * uval + vval * vval + wval * wval;
          if (dist > val) { idx = (unsigned)s; dist = val; }
        }
        tcon[ci] = (unsigned char)idx;
      }
      for (int r = 0; r < sz; r++) {
        const int tid1 = c.e[t][r], tid2 = c.e[t][(r + 1) % sz];
        const int cid1 = tcon[tid1], cid2 = tcon[tid2];
        int rr = (cid1 - cid2) < 0 ? cid2 - cid1 : cid1 - cid2;
        const int dst = rr > 2 ? 6 - rr : rr;
        if (dst == 0) {
          push_tri(st, vidx[tid1], vidx[tid2], tg[cid1]);
        } else if (dst == 1) {
          const double l1 = (e_vert(ecoord, tid1, 0) - hvt[cid2][0]) * (e_vert(ecoord, tid1, 0) - hvt[cid2][0]) +
                            (e_vert(ecoord, tid1, 1) - hvt[cid2][1]) * (e_vert(ecoord, tid1, 1) - hvt[cid2][1]) +
                            (e_vert(ecoord, tid1, 2) - hvt[cid2][2]) * (e_vert(ecoord, tid1, 2) - hvt[cid2][2]);
          const double l2 = (e_vert(ecoord, tid2, 0) - hvt[cid1][0]) * (e_vert(ecoord, tid2, 0) - hvt[cid1][0]) +
                            (e_vert(ecoord, tid2, 1) - hvt[cid1][1]) * (e_vert(ecoord, tid2, 1) - hvt[cid1][1]) +
                            (e_vert(ecoord, tid2, 2) - hvt[cid1][2]) * (e_vert(ecoord, tid2, 2) - hvt[cid1][2]);
          if (l1 < l2) {
            push_tri(st, vidx[tid1], vidx[tid2], tg[cid2]);
            push_tri(st, vidx[tid1], tg[cid2], tg[cid1]);
          } else {
            push_tri(st, vidx[tid1], vidx[tid2], tg[cid1]);
            push_tri(st, vidx[tid2], tg[cid2], tg[cid1]);
          }
        } else if (dst == 2) {
          const int dmax = (cid1 > cid2) ? cid1 : cid2, dmin = (cid1 < cid2) ? cid1 : cid2;
          const int cidm = ((dmax + 2) % 6 == dmin) ? (dmax + 1) % 6 : (dmax + dmin) / 2;
          push_tri(st, vidx[tid1], vidx[tid2], tg[cidm]);
          push_tri(st, vidx[tid1], tg[cidm], tg[cid1]);
          push_tri(st, vidx[tid2], tg[cid2], tg[cidm]);
        }
        /* a ring distance of 3 adds no triangle (no case in the reference's switch) */
      }
    }
    if (c.n == 1) {
      st->cases[8]--;
      st->cases[9]++;
      const int s_ = (og_decider(F[0], F[1], F[2], F[3]) <= i0);
      const int of_ = (wi[1] < wi[0]) ? s_ : !s_;
      if (!of_) {
        push_tri(st, tg[0], tg[2], tg[1]); push_tri(st, tg[2], tg[4], tg[3]);
        push_tri(st, tg[0], tg[5], tg[4]); push_tri(st, tg[0], tg[4], tg[2]);
      } else {
        push_tri(st, tg[0], tg[1], tg[2]); push_tri(st, tg[2], tg[3], tg[4]);
        push_tri(st, tg[0], tg[4], tg[5]); push_tri(st, tg[0], tg[2], tg[4]);
      }
    }
    return;
  }
  /* no tunnel (:1086-1299) */
  const unsigned nr_u = ((q_sol & 0x5) == 0x5) + ((q_sol & 0xA) == 0xA);
  const unsigned nr_v = ((q_sol & 0x11) == 0x11) + ((q_sol & 0x22) == 0x22);
  const unsigned nr_w = ((q_sol & 0x18) == 0x18) + ((q_sol & 0x24) == 0x24);
  const unsigned nr_t = nr_u + nr_v + nr_w;
  if (nr_t == nr_u || nr_t == nr_v || nr_t == nr_w) {
    for (int t = 0; t < c.n; t++) {
      const int* e = c.e[t];
      switch (c.size[t]) {
        case 3: push_tri(st, vidx[e[0]], vidx[e[1]], vidx[e[2]]); st->cases[0]++; break;
        case 4:
          push_tri(st, vidx[e[0]], vidx[e[1]], vidx[e[2]]);
          push_tri(st, vidx[e[0]], vidx[e[2]], vidx[e[3]]);
          st->cases[1]++;
          break;
        case 5:
          push_tri(st, vidx[e[0]], vidx[e[1]], vidx[e[2]]);
          push_tri(st, vidx[e[0]], vidx[e[2]], vidx[e[3]]);
          push_tri(st, vidx[e[0]], vidx[e[3]], vidx[e[4]]);
          st->cases[2]++;
          break;
        case 6:
          push_tri(st, vidx[e[0]], vidx[e[1]], vidx[e[3]]);
          push_tri(st, vidx[e[1]], vidx[e[2]], vidx[e[3]]);
          push_tri(st, vidx[e[0]], vidx[e[3]], vidx[e[4]]);
          push_tri(st, vidx[e[0]], vidx[e[4]], vidx[e[5]]);
          st->cases[3]++;
          break;
        default: break;
      }
    }
    return;
  }
  /* saddle points: one inner vertex (:1178-1296) */
  const unsigned fs[3][2] = {{q_sol & 1, (q_sol >> 1) & 1}, {(q_sol >> 2) & 1, (q_sol >> 3) & 1}, {(q_sol >> 4) & 1, (q_sol >> 5) & 1}};
  const unsigned fc1 = fs[0][0] * fs[1][0] + fs[0][1] * fs[1][1];
  const unsigned fc2 = fs[0][0] * fs[2][0] + fs[0][1] * fs[2][1];
  const unsigned fc3 = fs[1][0] * fs[2][1] + fs[1][1] * fs[2][0];
  const unsigned c_faces = fc1 + fc2 + fc3;
  double uc = 0, vc = 0, wc = 0;
  switch (c_faces) {
    case 2:
      if (fc1 == 0) {
        uc = fs[0][0] * ui[0] + fs[0][1] * ui[1]; vc = fs[1][0] * vi[0] + fs[1][1] * vi[1]; wc = fs[1][0] * wi[1] + fs[1][1] * wi[0];
      } else if (fc2 == 0) {
        uc = fs[0][0] * ui[0] + fs[0][1] * ui[1]; vc = fs[0][0] * vi[0] + fs[0][1] * vi[1]; wc = fs[0][0] * wi[1] + fs[0][1] * wi[0];
      } else if (fc3 == 0) {
        uc = fs[1][0] * ui[0] + fs[1][1] * ui[1]; vc = fs[1][0] * vi[0] + fs[1][1] * vi[1]; wc = fs[1][0] * wi[0] + fs[1][1] * wi[1];
      }
      break;
    case 3:
      uc = (fs[0][0] * ui[0] + fs[0][1] * ui[1]) / (int)(fs[0][0] + fs[0][1]);
      vc = (fs[1][0] * vi[0] + fs[1][1] * vi[1]) / (int)(fs[1][0] + fs[1][1]);
      wc = (fs[2][0] * wi[0] + fs[2][1] * wi[1]) / (int)(fs[2][0] + fs[2][1]);
      break;
    case 4: {
      const unsigned nu = fs[0][0] + fs[0][1], nv = fs[1][0] + fs[1][1], nw = fs[2][0] + fs[2][1];
      if (nw == 1) {
        uc = fs[2][0] * ui[0] + fs[2][1] * ui[1]; vc = fs[2][1] * vi[0] + fs[2][0] * vi[1]; wc = fs[2][0] * wi[0] + fs[2][1] * wi[1];
      } else if (nv == 1) {
        uc = fs[1][0] * ui[0] + fs[1][1] * ui[1]; vc = fs[1][0] * vi[0] + fs[1][1] * vi[1]; wc = fs[1][1] * wi[0] + fs[1][0] * wi[1];
      } else if (nu == 1) {
        uc = fs[0][0] * ui[0] + fs[0][1] * ui[1]; vc = fs[0][0] * vi[0] + fs[0][1] * vi[1]; wc = fs[0][0] * wi[0] + fs[0][1] * wi[1];
      }
    } break;
    default: break;
  }
  double ip[3], in[3];
  cell_trilinear(p, uc, vc, wc, ip);
  cell_trilinear(n, uc, vc, wc, in);
  const double factor = sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
  in[0] = in[0] / factor; in[1] = in[1] / factor; in[2] = in[2] / factor;
  const int g_index = (int)(st->pts.n / 3);
  int pt_used = 0;
  for (int t = 0; t < c.n; t++) {
    const int sz = c.size[t];
    if (sz == 3) {
      push_tri(st, vidx[c.e[t][0]], vidx[c.e[t][1]], vidx[c.e[t][2]]);
    } else {
      pt_used = 1;
      for (int r = 0; r < sz; r++) push_tri(st, vidx[c.e[t][r]], vidx[c.e[t][(r + 1) % sz]], g_index);
    }
  }
  if (pt_used) {
    for (int dd = 0; dd < 3; dd++) { og_dvec_push(&st->pts, ip[dd]); og_dvec_push(&st->nrm, in[dd]); }
  }
}

/* t_mc (mc/MarchingCubes.cpp:151-317) */
static void t_mc(tmc_state* st) {
  const og_grid* g = st->g;
  for (int k = 0; k < g->nz - 1; k++)
    for (int j = 0; j < g->ny - 1; j++)
      for (int i = 0; i < g->nx - 1; i++) {
        double u[8], p[8][3], n[8][3];
        unsigned ic = 0;
        int vi = 0;
        for (int kl = 0; kl <= 1; kl++)
          for (int jl = 0; jl <= 1; jl++)
            for (int il = 0; il <= 1; il++) {
              p[vi][0] = g->origin[0] + (i + il) * g->spacing[0];
              p[vi][1] = g->origin[1] + (j + jl) * g->spacing[1];
              p[vi][2] = g->origin[2] + (k + kl) * g->spacing[2];
              u[vi] = og_s(g, i + il, j + jl, k + kl);
              if (u[vi] >= st->i0) ic |= 1u << vi;
              const double* gr = st->grad + 3 * (((size_t)(k + kl) * g->ny + (j + jl)) * g->nx + (i + il));
              n[vi][0] = gr[0]; n[vi][1] = gr[1]; n[vi][2] = gr[2];
              vi++;
            }
        if (og_is_ambiguous(ic)) {
          p_slice(st, i, j, k, u, p, n, ic);
          continue;
        }
        int vidx[12];
        for (int e = 0; e < 12; e++)
          if (TMC_EDGE_MASK[ic] & (1u << e)) vidx[e] = edge_vertex(st, i, j, k, e, u, p, n, NULL);
        const int nt = og_tri_count(ic);
        for (int t = 0; t < nt; t++)
          push_tri(st, vidx[og_tri_edge(ic, t, 2)], vidx[og_tri_edge(ic, t, 1)], vidx[og_tri_edge(ic, t, 0)]);
      }
}

typedef struct { int64_t nv, nt; double* v; double* n; int* tris; int64_t cases[11]; } tmc_result;

void* oracle_tmc_run(int nx, int ny, int nz, const double* origin, const double* spacing, const float* field,
                     double iso, int key_bits) {
  og_grid g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  for (int d = 0; d < 3; d++) { g.origin[d] = origin[d]; g.spacing[d] = spacing[d]; }
  g.f = field;
  tmc_state st;
  memset(&st, 0, sizeof st);
  st.g = &g;
  st.i0 = iso;
  st.key_bits = key_bits;
  st.grad = tmc_gradient(&g);
  kmap_init(&st.map, 1024);
  t_mc(&st);
  free((void*)st.grad);
  free(st.map.keys); free(st.map.vals);
  tmc_result* r = (tmc_result*)calloc(1, sizeof(tmc_result));
  r->nv = (int64_t)(st.pts.n / 3);
  r->nt = (int64_t)(st.tris.n / 3);
  r->v = st.pts.a; r->n = st.nrm.a; r->tris = st.tris.a;
  memcpy(r->cases, st.cases, sizeof r->cases);
  return r;
}

void oracle_tmc_sizes(void* h, int64_t* out2) {
  tmc_result* r = (tmc_result*)h;
  out2[0] = r->nv; out2[1] = r->nt;
}

void oracle_tmc_copy(void* h, double* v, double* n, int* tris) {
  tmc_result* r = (tmc_result*)h;
  if (v && r->nv) memcpy(v, r->v, 3 * r->nv * sizeof(double));
  if (n && r->nv) memcpy(n, r->n, 3 * r->nv * sizeof(double));
  if (tris && r->nt) memcpy(tris, r->tris, 3 * r->nt * sizeof(int));
}

void oracle_tmc_cases(void* h, int64_t* out11) {
  tmc_result* r = (tmc_result*)h;
  memcpy(out11, r->cases, sizeof r->cases);
}

void oracle_tmc_free(void* h) {
  tmc_result* r = (tmc_result*)h;
  free(r->v); free(r->n); free(r->tris); free(r);
}
