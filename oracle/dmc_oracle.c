/* CPU oracle for Dual Marching Cubes -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's single-threaded CPU path
 * dmc::DualMarchingCubes::dualMC (cpp_dmc/DualMarchingCubes.cpp:5-88): cell classification,
 * MC polygons with the asymptotic decider, the sampled vertex representative, quads keyed by the
 * dual grid edge and collected in key order, unused-vertex removal, P3X3Y (colour pass and
 * isolated pass) and P3333 simplification, halfedges and the quad->triangle split.  Mixed
 * float/double arithmetic is kept exactly as the reference writes it, so results are bit-equal
 * when both are compiled with -ffp-contract=off.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load this library.
 */
#include <math.h>
#include <stdio.h>

#include "oracle_common.h"

#define INVALID (-1)
#define MANIFOLD 0
#define NON_MANIFOLD 1
#define BOUNDARY_MULTIPLE_EDGE 2

typedef struct { double x[3]; } vec3;

typedef struct {
  int64_t nv, nq, nt, nhe;
  double* v;
  double* n;
  int* quads;
  int* tris;
  int* he; /* 5 ints per halfedge: origin, face, next, twin, manifold flag */
  int* he_v;
  int* he_f;
  int* colors;    /* front only: inherited quad colours */
  int64_t* vcell; /* front only: generating cell of each vertex */
  float* vuvw;    /* front only: local coordinates of each vertex */
  int64_t proj_fail[2];
} dmc_result;

/* ---------------------------------------------------------------------------------------- */
/* gradient: UniformGrid::estimateGradient (cpp_dmc/UniformGrid.cpp:512-540) incl. its upper  */
/* border rule index(i+1) -> max - (i+1) = 0, and flip_gradient (:542-553)                   */
/* ---------------------------------------------------------------------------------------- */
static int grad_index(int i, int max) { return (i < 0) ? 0 : (i >= max) ? max - i : i; }

static double* estimate_gradient(const og_grid* g, int flip) {
  const size_t nr = (size_t)g->nx * g->ny * g->nz;
  double* gr = (double*)malloc(3 * nr * sizeof(double));
  for (size_t s = 0; s < nr; s++) {
    const int i = (int)(s % g->nx), j = (int)((s / g->nx) % g->ny), k = (int)(s / ((size_t)g->nx * g->ny));
    const int i0 = grad_index(i - 1, g->nx), i1 = grad_index(i + 1, g->nx);
    const int j0 = grad_index(j - 1, g->ny), j1 = grad_index(j + 1, g->ny);
    const int k0 = grad_index(k - 1, g->nz), k1 = grad_index(k + 1, g->nz);
    double nx = (og_s(g, i1, j, k) - og_s(g, i0, j, k)) / (2 * g->spacing[0]);
    double ny = (og_s(g, i, j1, k) - og_s(g, i, j0, k)) / (2 * g->spacing[1]);
    double nz = (og_s(g, i, j, k1) - og_s(g, i, j, k0)) / (2 * g->spacing[2]);
    if (flip) { nx *= -1.; ny *= -1.; nz *= -1.; }
    gr[3 * s] = nx; gr[3 * s + 1] = ny; gr[3 * s + 2] = nz;
  }
  return gr;
}

/* ---------------------------------------------------------------------------------------- */
/* MC polygon with the decider, DMC variant (>= isovalue): mc_polygon(i0, F, c_)             */
/* (cpp_dmc/DualMarchingCubes.cpp:328-467)                                                   */
/* ---------------------------------------------------------------------------------------- */
static void dmc_polygon_ambiguous(double i0, const double F[8], og_contours* c) {
  int to[12];
  for (int e = 0; e < 12; e++) to[e] = -1;
  for (int f = 0; f < 6; f++) {
    const int* fv = OG_FACE_V[f];
    const double f0 = F[fv[0]], f1 = F[fv[1]], f2 = F[fv[2]], f3 = F[fv[3]];
    int fc = 0;
    if (f0 >= i0) fc |= 1;
    if (f1 >= i0) fc |= 2;
    if (f2 >= i0) fc |= 4;
    if (f3 >= i0) fc |= 8;
    int sep = 0;
    if (fc == 6 || fc == 9) {
      const double val = og_decider(f0, f1, f2, f3);
      if (val >= i0) sep = 1;
      else if (val < i0) sep = 0;
      else continue; /* NaN: the reference sets no segment */
    }
    og_face_rule(fc, sep, OG_FACE_E[f], to);
  }
  og_connect(to, c);
}

/* getLocalCoordinates (cpp_dmc/DualMarchingCubes.h:391-407): float edge parameter, float ops */
static void local_coord(int e, const double f[8], double i0, double u[3]) {
  const int v0 = OG_EDGE_V[e][0], v1 = OG_EDGE_V[e][1];
  const float l = (i0 - f[v0]) / (f[v1] - f[v0]);
  for (int d = 0; d < 3; d++) {
    const float val = (float)OG_EDGE_DIR[e][d];
    const float con = (float)OG_EDGE_CON[e][d];
    u[d] = l * val + con;
  }
}

typedef struct { double b[4][2]; } bbox1;

/* isInNeighborBBox (cpp_dmc/DualMarchingCubes.h:498-517) */
static int in_neighbor_bbox(double u, double v, double w, int cnt, const og_contours* c, int t,
                            const bbox1* bU, const bbox1* bV, const bbox1* bW) {
  for (int i = 0; i < cnt; i++) {
    if (c->size[i] == 3 && t != i) {
      if (u < bU->b[i][0] || bU->b[i][1] < u) continue;
      if (v < bV->b[i][0] || bV->b[i][1] < v) continue;
      if (w < bW->b[i][0] || bW->b[i][1] < w) continue;
      return 1;
    }
  }
  return 0;
}

/* vertex permutations of the three projection planes: w_proj, v_proj, u_proj
 * (cpp_dmc/DualMarchingCubes.cpp:198-200); entries 1..7 of each */
static const int PROJ_V[3][8] = {{0, 1, 2, 3, 4, 5, 6, 7}, {0, 1, 4, 5, 2, 3, 6, 7}, {0, 2, 4, 6, 1, 3, 5, 7}};

/* projection (cpp_dmc/DualMarchingCubes.cpp:274-326) */
static int projection(int pr, double i0, const double f[8], int cnt, const og_contours* c, int t, double p[3],
                      const bbox1* bU, const bbox1* bV, const bbox1* bW, int nrSamples) {
  const int* r = PROJ_V[pr];
  const double umin = bU->b[t][0], umax = bU->b[t][1];
  const double vmin = bV->b[t][0], vmax = bV->b[t][1];
  const double du = (umax - umin) / (nrSamples - 1);
  const double dv = (vmax - vmin) / (nrSamples - 1);
  double minDistance = 100;
  double pt[3] = {0, 0, -1};
  double wmin = bW->b[t][0], wmax = bW->b[t][1];
  const double eps = 1e-5;
  if (fabs(wmax - wmin) < eps) { wmin -= eps; wmax += eps; }
  const int cnt_size = c->size[t];
  for (int i = 1; i < (nrSamples - 1); i++) {
    const float u = umin + i * du;
    for (int j = 1; j < (nrSamples - 1); j++) {
      const float v = vmin + j * dv;
      const float g1 = (1 - v) * ((1 - u) * f[0] + u * f[r[1]]) + v * ((1 - u) * f[r[2]] + u * f[r[3]]);
      const float g2 = (1 - v) * ((1 - u) * f[r[4]] + u * f[r[5]]) + v * ((1 - u) * f[r[6]] + u * f[r[7]]);
      if (g1 == g2) continue;
      const float w = (i0 - g1) / (g2 - g1);
      if (wmin <= w && w <= wmax) {
        if (cnt == 1 || cnt_size == 3 || !in_neighbor_bbox(u, v, w, cnt, c, t, bU, bV, bW)) {
          const float d = (p[0] - u) * (p[0] - u) + (p[1] - v) * (p[1] - v) + (p[2] - w) * (p[2] - w);
          if (minDistance > d) {
            minDistance = d;
            pt[0] = u; pt[1] = v; pt[2] = w;
          }
        }
      }
    }
  }
  if (pt[2] > -1) { p[0] = pt[0]; p[1] = pt[1]; p[2] = pt[2]; return 1; }
  return 0;
}

/* trilinear gradient of the cell (cpp_dmc/DualMarchingCubes.h:580-587) */
static void cell_gradient(const double f[8], double u, double v, double w, double g[3]) {
  g[0] = (1 - w) * ((1 - v) * (f[1] - f[0]) + v * (f[3] - f[2])) + w * ((1 - v) * (f[5] - f[4]) + v * (f[7] - f[6]));
  g[1] = (1 - w) * ((1 - u) * (f[2] - f[0]) + u * (f[3] - f[1])) + w * ((1 - u) * (f[6] - f[4]) + u * (f[7] - f[5]));
  g[2] = (1 - v) * ((1 - u) * (f[4] - f[0]) + u * (f[5] - f[1])) + v * ((1 - u) * (f[6] - f[2]) + u * (f[7] - f[3]));
}

/* representative (cpp_dmc/DualMarchingCubes.cpp:194-272) */
static void representative(double i0, const double f[8], int cnt, const og_contours* c, int t, double p[3],
                           const bbox1* bU, const bbox1* bV, const bbox1* bW, int64_t* fail) {
  const int nrSamples = 9;
  int prj = 0; /* 0 = W, 1 = V, 2 = U projection */
  if (c->size[t] >= 6) {
    double ni[3];
    cell_gradient(f, p[0], p[1], p[2], ni);
    const double dx = fabs(ni[0]), dy = fabs(ni[1]), dz = fabs(ni[2]);
    if (dz >= dx && dz >= dy) prj = 0;
    else if (dy >= dx && dy >= dz) prj = 1;
    else if (dx >= dy && dx >= dz) prj = 2;
    else prj = 0;
  } else {
    const double u = bU->b[t][1] - bU->b[t][0], v = bV->b[t][1] - bV->b[t][0], w = bW->b[t][1] - bW->b[t][0];
    if (w <= u && w <= v) prj = 0;
    else if (v <= u && v <= w) prj = 1;
    else if (u <= v && u <= w) prj = 2;
    else prj = 0;
  }
  double pt[3];
  if (prj == 0) {
    pt[0] = p[0]; pt[1] = p[1]; pt[2] = p[2];
    if (!projection(0, i0, f, cnt, c, t, pt, bU, bV, bW, nrSamples)) {
      fail[0]++;
      if (!projection(0, i0, f, cnt, c, t, pt, bU, bV, bW, nrSamples * 3 + 1)) fail[1]++;
    }
    p[0] = pt[0]; p[1] = pt[1]; p[2] = pt[2];
  } else if (prj == 1) {
    pt[0] = p[0]; pt[1] = p[2]; pt[2] = p[1];
    if (!projection(1, i0, f, cnt, c, t, pt, bU, bW, bV, nrSamples)) {
      fail[0]++;
      if (!projection(1, i0, f, cnt, c, t, pt, bU, bW, bV, nrSamples * 3 + 1)) fail[1]++;
    }
    p[0] = pt[0]; p[1] = pt[2]; p[2] = pt[1];
  } else {
    pt[0] = p[1]; pt[1] = p[2]; pt[2] = p[0];
    if (!projection(2, i0, f, cnt, c, t, pt, bV, bW, bU, nrSamples)) {
      fail[0]++;
      if (!projection(2, i0, f, cnt, c, t, pt, bV, bW, bU, nrSamples * 3 + 1)) fail[1]++;
    }
    p[0] = pt[2]; p[1] = pt[0]; p[2] = pt[1];
  }
}

/* ---------------------------------------------------------------------------------------- */
/* front end: dualMC cell loop + slice + collectQuadrilaterals + removeUnusedVertices          */
/* ---------------------------------------------------------------------------------------- */
typedef struct { int key; int pos; int v; int color; int seq; } qentry;
OG_VEC(qvec, qentry)

static int cmp_qentry(const void* a, const void* b) {
  const qentry* x = (const qentry*)a; const qentry* y = (const qentry*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

typedef struct {
  og_dvec v, n;    /* 3 per vertex */
  og_ivec quads;   /* 4 per quad */
  og_ivec colors;  /* per quad */
  og_lvec vcell;
  og_fvec vuvw;
} mesh_t;

/* dualMC cell loop (cpp_dmc/DualMarchingCubes.cpp:16-50) and slice (:97-192) */
static void dmc_front(const og_grid* g, const double* grad, double i0, mesh_t* m, int64_t fail[2]) {
  qvec entries = {0};
  const int idim = g->nx, jdim = g->ny, kdim = g->nz;
  for (int k = 0; k < kdim - 1; k++)
    for (int j = 0; j < jdim - 1; j++)
      for (int i = 0; i < idim - 1; i++) {
        double u[8];
        u[0] = og_s(g, i, j, k); u[1] = og_s(g, i + 1, j, k);
        u[2] = og_s(g, i, j + 1, k); u[3] = og_s(g, i + 1, j + 1, k);
        u[4] = og_s(g, i, j, k + 1); u[5] = og_s(g, i + 1, j, k + 1);
        u[6] = og_s(g, i, j + 1, k + 1); u[7] = og_s(g, i + 1, j + 1, k + 1);
        unsigned cs = 0;
        for (int b = 0; b < 8; b++) cs += ((unsigned)(u[b] >= i0)) << b;
        if (cs == 0 || cs == 255) continue;
        /* slice */
        og_contours c;
        if (og_is_ambiguous(cs)) dmc_polygon_ambiguous(i0, u, &c);
        else og_table_contour(cs, &c);
        bbox1 bU, bV, bW;
        memset(&bU, 0, sizeof bU); memset(&bV, 0, sizeof bV); memset(&bW, 0, sizeof bW);
        unsigned e_bits = 0;
        for (int t = 0; t < c.n; t++) {
          bU.b[t][0] = 1; bU.b[t][1] = 0; bV.b[t][0] = 1; bV.b[t][1] = 0; bW.b[t][0] = 1; bW.b[t][1] = 0;
          for (int q = 0; q < c.size[t]; q++) {
            const int e = c.e[t][q];
            double ui[3];
            local_coord(e, u, i0, ui);
            bU.b[t][0] = bU.b[t][0] > ui[0] ? ui[0] : bU.b[t][0];
            bU.b[t][1] = bU.b[t][1] < ui[0] ? ui[0] : bU.b[t][1];
            bV.b[t][0] = bV.b[t][0] > ui[1] ? ui[1] : bV.b[t][0];
            bV.b[t][1] = bV.b[t][1] < ui[1] ? ui[1] : bV.b[t][1];
            bW.b[t][0] = bW.b[t][0] > ui[2] ? ui[2] : bW.b[t][0];
            bW.b[t][1] = bW.b[t][1] < ui[2] ? ui[2] : bW.b[t][1];
            if (u[OG_EDGE_V[e][0]] < i0) e_bits |= (1u << e);
          }
        }
        for (int t = 0; t < c.n; t++) {
          const int cnt_size = c.size[t];
          double p[3] = {0, 0, 0};
          for (int q = 0; q < cnt_size; q++) {
            double ui[3];
            local_coord(c.e[t][q], u, i0, ui);
            p[0] += ui[0]; p[1] += ui[1]; p[2] += ui[2];
          }
          p[0] /= cnt_size; p[1] /= cnt_size; p[2] /= cnt_size;
          representative(i0, u, c.n, &c, t, p, &bU, &bV, &bW, fail);
          /* UniformGrid::normal (cpp_dmc/UniformGrid.h:286-298) */
          double nv[3];
          {
            const double uu = p[0], vv = p[1], ww = p[2];
            const double* G[8];
            G[0] = grad + 3 * ((size_t)og_gindex(g, i, j, k));
            G[1] = grad + 3 * ((size_t)og_gindex(g, i + 1, j, k));
            G[2] = grad + 3 * ((size_t)og_gindex(g, i, j + 1, k));
            G[3] = grad + 3 * ((size_t)og_gindex(g, i + 1, j + 1, k));
            G[4] = grad + 3 * ((size_t)og_gindex(g, i, j, k + 1));
            G[5] = grad + 3 * ((size_t)og_gindex(g, i + 1, j, k + 1));
            G[6] = grad + 3 * ((size_t)og_gindex(g, i, j + 1, k + 1));
            G[7] = grad + 3 * ((size_t)og_gindex(g, i + 1, j + 1, k + 1));
            for (int d = 0; d < 3; d++) {
              nv[d] = (1 - ww) * ((1 - vv) * ((1 - uu) * G[0][d] + uu * G[1][d]) + vv * ((1 - uu) * G[2][d] + uu * G[3][d])) +
                      ww * ((1 - vv) * ((1 - uu) * G[4][d] + uu * G[5][d]) + vv * ((1 - uu) * G[6][d] + uu * G[7][d]));
            }
            const double s_ = sqrt(nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2]);
            nv[0] /= s_; nv[1] /= s_; nv[2] /= s_;
          }
          /* UniformGrid::position (cpp_dmc/UniformGrid.h:300-305) */
          double pi[3];
          pi[0] = g->origin[0] + (i + p[0]) * g->spacing[0];
          pi[1] = g->origin[1] + (j + p[1]) * g->spacing[1];
          pi[2] = g->origin[2] + (k + p[2]) * g->spacing[2];
          const int v_addr = (int)(m->v.n / 3);
          for (int d = 0; d < 3; d++) { og_dvec_push(&m->v, pi[d]); og_dvec_push(&m->n, nv[d]); }
          og_lvec_push(&m->vcell, (int64_t)i + (int64_t)(idim - 1) * ((int64_t)j + (int64_t)(jdim - 1) * k));
          for (int d = 0; d < 3; d++) og_fvec_push(&m->vuvw, (float)p[d]);
          for (int q = 0; q < cnt_size; q++) {
            const int e = c.e[t][q];
            const int gi = i + OG_EDGE_GLOBAL[e][0], gj = j + OG_EDGE_GLOBAL[e][1], gk = k + OG_EDGE_GLOBAL[e][2];
            const int key = 3 * og_gindex(g, gi, gj, gk) + OG_EDGE_GLOBAL[e][3];
            const int pos = OG_QUAD_SLOT[e][(e_bits >> e) & 1];
            int color = -1;
            const int par = (i & 1) | (j & 1) << 1 | (k & 1) << 2;
            if (e == 0) color = 3 * par;
            if (e == 3) color = 3 * par + 1;
            if (e == 8) color = 3 * par + 2;
            qentry qe = {key, pos, v_addr, color, (int)entries.n};
            qvec_push(&entries, qe);
          }
        }
      }
  /* collectQuadrilaterals: std::map in key order (cpp_dmc/DualMarchingCubes.h:607-676) */
  qsort(entries.a, entries.n, sizeof(qentry), cmp_qentry);
  for (size_t s = 0; s < entries.n;) {
    size_t e = s;
    int q[5] = {INVALID, INVALID, INVALID, INVALID, -1};
    while (e < entries.n && entries.a[e].key == entries.a[s].key) {
      q[entries.a[e].pos] = entries.a[e].v;
      if (entries.a[e].color != -1) q[4] = entries.a[e].color;
      e++;
    }
    if (q[0] != INVALID && q[1] != INVALID && q[2] != INVALID && q[3] != INVALID) {
      for (int d = 0; d < 4; d++) og_ivec_push(&m->quads, q[d]);
      og_ivec_push(&m->colors, q[4]);
    }
    s = e;
  }
  qvec_free(&entries);
  /* removeUnusedVertices (cpp_dmc/DualMarchingCubes.h:685-729) */
  const size_t nr_v = m->v.n / 3, nr_q = m->quads.n / 4;
  char* flag = (char*)calloc(nr_v + 1, 1);
  for (size_t f = 0; f < 4 * nr_q; f++) flag[m->quads.a[f]] = 1;
  int* mp = (int*)malloc((nr_v + 1) * sizeof(int));
  size_t w = 0;
  for (size_t i = 0; i < nr_v; i++) {
    mp[i] = INVALID;
    if (flag[i]) {
      mp[i] = (int)w;
      for (int d = 0; d < 3; d++) { m->v.a[3 * w + d] = m->v.a[3 * i + d]; m->n.a[3 * w + d] = m->n.a[3 * i + d]; m->vuvw.a[3 * w + d] = m->vuvw.a[3 * i + d]; }
      m->vcell.a[w] = m->vcell.a[i];
      w++;
    }
  }
  m->v.n = 3 * w; m->n.n = 3 * w; m->vuvw.n = 3 * w; m->vcell.n = w;
  for (size_t f = 0; f < 4 * nr_q; f++) m->quads.a[f] = mp[m->quads.a[f]];
  free(flag); free(mp);
}

/* ---------------------------------------------------------------------------------------- */
/* halfedges (cpp_dmc/DualMarchingCubes.cpp:488-671)                                         */
/* ---------------------------------------------------------------------------------------- */
typedef struct { uint64_t key; int he; } hkey;
static int cmp_hkey(const void* a, const void* b) {
  const hkey* x = (const hkey*)a; const hkey* y = (const hkey*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->he < y->he ? -1 : (x->he > y->he);
}
static uint64_t he_key(int v0, int v1) {
  if (v0 < v1) return ((uint64_t)(unsigned)v0 << 32) | ((uint64_t)(unsigned)v1 & 0xffffffffull);
  return ((uint64_t)(unsigned)v1 << 32) | ((uint64_t)(unsigned)v0 & 0xffffffffull);
}

typedef struct { int* he; int* hv; int* hf; int nq; int nv; } hmesh;

static void halfedges_p(int nr_v, const int* quads, int P, int nr_q, hmesh* h) {
  h->nq = nr_q; h->nv = nr_v;
  h->he = (int*)malloc((size_t)5 * P * nr_q * sizeof(int) + 1);
  h->hv = (int*)malloc((size_t)nr_v * sizeof(int) + 1);
  h->hf = (int*)malloc((size_t)nr_q * sizeof(int) + 1);
  for (int v = 0; v < nr_v; v++) h->hv[v] = INVALID;
  hkey* keys = (hkey*)malloc((size_t)P * nr_q * sizeof(hkey) + 1);
  for (int i = 0; i < nr_q; i++) {
    const int* q = quads + P * i;
    for (int r = 0; r < P; r++) {
      int* e = h->he + 5 * (P * i + r);
      e[0] = q[r]; e[1] = i; e[2] = P * i + (r + 1) % P; e[3] = INVALID; e[4] = MANIFOLD;
    }
    h->hf[i] = P * i;
    for (int r = 0; r < P; r++) h->hv[q[r]] = P * i + r;
    for (int r = 0; r < P; r++) { keys[P * i + r].key = he_key(q[r], q[(r + 1) % P]); keys[P * i + r].he = P * i + r; }
  }
  qsort(keys, (size_t)P * nr_q, sizeof(hkey), cmp_hkey);
#define HE(x) (h->he + 5 * (size_t)(x))
  for (size_t s = 0; s < (size_t)P * nr_q;) {
    size_t t = s;
    while (t < (size_t)P * nr_q && keys[t].key == keys[s].key) t++;
    const int c = (int)(t - s);
    if (c == 1) {
      HE(keys[s].he)[3] = INVALID;
    } else if (c == 2) {
      const int e0 = keys[s].he, e1 = keys[s + 1].he;
      HE(e0)[3] = e1; HE(e1)[3] = e0;
    } else if (c == 3) {
      const int e0 = keys[s].he, e1 = keys[s + 1].he, e2 = keys[s + 2].he;
      const int v0 = HE(e0)[0], v1 = HE(e1)[0], v2 = HE(e2)[0];
      HE(e0)[4] = BOUNDARY_MULTIPLE_EDGE; HE(e1)[4] = BOUNDARY_MULTIPLE_EDGE; HE(e2)[4] = BOUNDARY_MULTIPLE_EDGE;
      if (v0 != v1) { HE(e0)[3] = e1; HE(e1)[3] = e0; HE(e2)[3] = INVALID; h->hv[v2] = e2; }
      else if (v0 != v2) { HE(e0)[3] = e2; HE(e2)[3] = e0; HE(e1)[3] = INVALID; h->hv[v1] = e1; }
      else { HE(e1)[3] = e2; HE(e2)[3] = e1; HE(e0)[3] = INVALID; h->hv[v0] = e0; }
    } else if (c == 4) {
      const int e0 = keys[s].he, e1 = keys[s + 1].he, e2 = keys[s + 2].he, e3 = keys[s + 3].he;
      const int v0 = HE(e0)[0], v1 = HE(e1)[0];
      if (v0 != v1) { HE(e0)[3] = e1; HE(e1)[3] = e0; HE(e2)[3] = e3; HE(e3)[3] = e2; }
      else { HE(e0)[3] = e2; HE(e2)[3] = e0; HE(e1)[3] = e3; HE(e3)[3] = e1; }
      HE(e0)[4] = NON_MANIFOLD; HE(e1)[4] = NON_MANIFOLD; HE(e2)[4] = NON_MANIFOLD; HE(e3)[4] = NON_MANIFOLD;
    } else {
      /* more than four faces at an edge: the reference records the first four in its
       * bucket and prints an error; only the first four halfedges get their fields touched,
       * and none of them changes here. */
    }
    s = t;
  }
#undef HE
  free(keys);
}
static void halfedges(int nr_v, const int* quads, int nr_q, hmesh* h) { halfedges_p(nr_v, quads, 4, nr_q, h); }
static void hmesh_free(hmesh* h) { free(h->he); free(h->hv); free(h->hf); }

#define HE(h, x) ((h)->he + 5 * (size_t)(x))

/* collectNeighbors (cpp_dmc/DualMarchingCubes.cpp:673-702) */
static void neighbors(const hmesh* h, int q, int n[4]) {
  const int e0 = h->hf[q], e1 = HE(h, e0)[2], e2 = HE(h, e1)[2], e3 = HE(h, e2)[2];
  const int t[4] = {HE(h, e0)[3], HE(h, e1)[3], HE(h, e2)[3], HE(h, e3)[3]};
  for (int r = 0; r < 4; r++) n[r] = (t[r] != INVALID) ? HE(h, t[r])[1] : -1;
}

/* isNonManifold (cpp_dmc/DualMarchingCubes.cpp:874-885) */
static int non_manifold(const hmesh* h, int f) {
  const int e0 = h->hf[f], e1 = HE(h, e0)[2], e2 = HE(h, e1)[2], e3 = HE(h, e2)[2];
  return HE(h, e0)[4] == NON_MANIFOLD || HE(h, e1)[4] == NON_MANIFOLD || HE(h, e2)[4] == NON_MANIFOLD ||
         HE(h, e3)[4] == NON_MANIFOLD;
}

/* pick the lowest colour in 0..lim not used by the four neighbours; -1 when none is free */
static int free_color(const int nc[4], int lim) {
  for (int col = 0; col <= lim; col++)
    if (nc[0] != col && nc[1] != col && nc[2] != col && nc[3] != col) return col;
  return -1;
}

/* colorFaces (cpp_dmc/DualMarchingCubes.cpp:714-844): the per-class face lists are taken from
 * the inherited colours before any reduction; fColor4 likewise holds the faces whose inherited
 * colour is 4. */
static void color_faces_full(const hmesh* h, int* colors) {
  const int nr_q = h->nq;
  og_ivec c4 = {0};
  for (int f = 0; f < nr_q; f++) if (colors[f] == 4) og_ivec_push(&c4, f);
  /* class lists are taken before any reduction: a face enters class c iff its colour was c */
  og_ivec cls_list[19];
  memset(cls_list, 0, sizeof cls_list);
  for (int f = 0; f < nr_q; f++) if (colors[f] > 4) og_ivec_push(&cls_list[colors[f] - 5], f);
  for (int c = 0; c < 19; c++) {
    for (size_t s = 0; s < cls_list[c].n; s++) {
      const int f = cls_list[c].a[s];
      int n[4], nc[4];
      neighbors(h, f, n);
      for (int r = 0; r < 4; r++) nc[r] = (n[r] != INVALID) ? colors[n[r]] : -1;
      const int col = free_color(nc, 4);
      if (col >= 0) colors[f] = col;
    }
    og_ivec_free(&cls_list[c]);
  }
  for (size_t s = 0; s < c4.n; s++) {
    const int f = c4.a[s];
    int n[4], nc[4];
    neighbors(h, f, n);
    for (int r = 0; r < 4; r++) nc[r] = (n[r] != INVALID) ? colors[n[r]] : -1;
    const int col = free_color(nc, 3);
    if (col >= 0) colors[f] = col;
  }
  og_ivec_free(&c4);
}

/* vertexValence (cpp_dmc/DualMarchingCubes.cpp:847-871) */
static int* vertex_valence(const hmesh* h) {
  int* vV = (int*)calloc((size_t)h->nv + 1, sizeof(int));
  for (int e = 0; e < 4 * h->nq; e++) {
    vV[HE(h, e)[0]]++;
    if (HE(h, e)[3] == INVALID) vV[HE(h, HE(h, e)[2])[0]]++;
  }
  return vV;
}

/* mark3X3Y (cpp_dmc/DualMarchingCubes.cpp:889-913) */
static char* mark3x3y(const int* quads, int nr_q, const int* vV) {
  char* p = (char*)calloc((size_t)nr_q + 1, 1);
  for (int f = 0; f < nr_q; f++) {
    const int a = vV[quads[4 * f]], b = vV[quads[4 * f + 1]], c = vV[quads[4 * f + 2]], d = vV[quads[4 * f + 3]];
    if ((a == 3 && b >= 5 && c == 3 && d >= 5) || (a >= 5 && b == 3 && c >= 5 && d == 3)) p[f] = 1;
  }
  return p;
}

static void merge_vertex(double* v, double* n, int dst, int a, int b) {
  for (int d = 0; d < 3; d++) v[3 * dst + d] = v[3 * a + d] + 0.5 * (v[3 * b + d] - v[3 * a + d]);
  for (int d = 0; d < 3; d++) n[3 * dst + d] = n[3 * a + d] + 0.5 * (n[3 * b + d] - n[3 * a + d]);
  const double s_ = sqrt(n[3 * dst] * n[3 * dst] + n[3 * dst + 1] * n[3 * dst + 1] + n[3 * dst + 2] * n[3 * dst + 2]);
  n[3 * dst] /= s_; n[3 * dst + 1] /= s_; n[3 * dst + 2] /= s_;
}

/* mergeVertices3X3Y, colour variant (cpp_dmc/DualMarchingCubes.cpp:916-1012) when colors != NULL,
 * isolated variant (:1014-1094) otherwise.  vm_first/vm_second/em are outputs. */
static void merge3x3y(double* v, double* nrm, const char* p, const int* vV, const int* colors, const hmesh* h,
                      char* vm_first, int* vm_second, char* em) {
  const int nr_q = h->nq;
  for (int i = 0; i < h->nv; i++) { vm_first[i] = 0; vm_second[i] = INVALID; }
  for (int f = 0; f < nr_q; f++) em[f] = 0;
  for (int f = 0; f < nr_q; f++) {
    if (!p[f]) continue;
    const int e0 = h->hf[f], e1 = HE(h, e0)[2], e2 = HE(h, e1)[2], e3 = HE(h, e2)[2];
    int n[4];
    neighbors(h, f, n);
    if (colors) {
      const int c = colors[f];
      int bad = 0;
      for (int r = 0; r < 4; r++) {
        if (n[r] >= 0 && non_manifold(h, n[r])) bad = 1;
        if (n[r] < 0) bad = 1;
      }
      if (bad) continue;
      int ok = 1;
      for (int r = 0; r < 4; r++) {
        int ncol = -1, npat = 0;
        if (n[r] != INVALID) { ncol = colors[n[r]]; npat = p[n[r]]; }
        if (npat && ncol <= c) ok = 0;
      }
      if (!ok) continue;
    } else {
      int skip = 0;
      for (int r = 0; r < 4; r++) if (n[r] != INVALID && non_manifold(h, n[r])) skip = 1;
      if (skip) continue;
      for (int r = 0; r < 4; r++) if (n[r] != INVALID && p[n[r]]) skip = 1;
      if (skip) continue;
    }
    const int v0 = HE(h, e0)[0], v1 = HE(h, e1)[0], v2 = HE(h, e2)[0], v3 = HE(h, e3)[0];
    const int a = vV[v0], b = vV[v1], c2 = vV[v2], d = vV[v3];
    if (a == 3 && b >= 5 && c2 == 3 && d >= 5) {
      merge_vertex(v, nrm, v0, v1, v3);
      vm_first[v2] = 1; vm_second[v2] = v0; em[f] = 1;
    } else if (a >= 5 && b == 3 && c2 >= 5 && d == 3) {
      merge_vertex(v, nrm, v1, v0, v2);
      vm_first[v3] = 1; vm_second[v3] = v1; em[f] = 1;
    }
  }
}

/* removeVertices3X3Y + removeQuadrilaterals3X3Y (cpp_dmc/DualMarchingCubes.cpp:1096-1137) */
static void remove3x3y(mesh_t* m, const char* vm_first, int* vm_second, const char* em) {
  const size_t nr_v = m->v.n / 3, nr_q = m->quads.n / 4;
  size_t w = 0;
  for (size_t i = 0; i < nr_v; i++) {
    if (!vm_first[i]) {
      for (int d = 0; d < 3; d++) { m->v.a[3 * w + d] = m->v.a[3 * i + d]; m->n.a[3 * w + d] = m->n.a[3 * i + d]; }
      vm_second[i] = (int)w;
      w++;
    }
  }
  m->v.n = 3 * w; m->n.n = 3 * w;
  size_t wq = 0;
  int* nq = (int*)malloc(m->quads.n * sizeof(int) + 1);
  for (size_t f = 0; f < nr_q; f++) {
    if (em[f]) continue;
    for (int r = 0; r < 4; r++) {
      const int vv = m->quads.a[4 * f + r];
      nq[4 * wq + r] = vm_first[vv] ? vm_second[vm_second[vv]] : vm_second[vv];
    }
    wq++;
  }
  memcpy(m->quads.a, nq, 4 * wq * sizeof(int));
  m->quads.n = 4 * wq;
  free(nq);
}

/* simplify3X3Y (cpp_dmc/DualMarchingCubes.cpp:1139-1182) */
static void simplify3x3y(mesh_t* m) {
  for (int pass = 0; pass < 2; pass++) {
    const int nr_v = (int)(m->v.n / 3), nr_q = (int)(m->quads.n / 4);
    hmesh h;
    halfedges(nr_v, m->quads.a, nr_q, &h);
    if (pass == 0) color_faces_full(&h, m->colors.a);
    int* vV = vertex_valence(&h);
    char* p = mark3x3y(m->quads.a, nr_q, vV);
    char* vm_first = (char*)calloc((size_t)nr_v + 1, 1);
    int* vm_second = (int*)malloc(((size_t)nr_v + 1) * sizeof(int));
    char* em = (char*)calloc((size_t)nr_q + 1, 1);
    merge3x3y(m->v.a, m->n.a, p, vV, pass == 0 ? m->colors.a : NULL, &h, vm_first, vm_second, em);
    remove3x3y(m, vm_first, vm_second, em);
    free(vV); free(p); free(vm_first); free(vm_second); free(em);
    hmesh_free(&h);
  }
}

/* mark3333, removeVertices3333, removeQuadrilaterals3333, simplify3333
 * (cpp_dmc/DualMarchingCubes.cpp:1189-1385) */
static void simplify3333(mesh_t* m) {
  const int nr_v = (int)(m->v.n / 3), nr_q = (int)(m->quads.n / 4);
  hmesh h;
  halfedges(nr_v, m->quads.a, nr_q, &h);
  int* vV = vertex_valence(&h);
  char* p = (char*)calloc((size_t)nr_q + 1, 1);
  char* rf = (char*)calloc((size_t)nr_q + 1, 1);
  char* vm0 = (char*)calloc((size_t)nr_v + 1, 1);
  int* vm1 = (int*)malloc(((size_t)nr_v + 1) * sizeof(int));
  int* vm2 = (int*)malloc(((size_t)nr_v + 1) * sizeof(int));
  for (int i = 0; i < nr_v; i++) { vm1[i] = -1; vm2[i] = -1; }
  for (int f = 0; f < nr_q; f++) {
    if (non_manifold(&h, f)) continue;
    const int e[4] = {h.hf[f], HE(&h, h.hf[f])[2], HE(&h, HE(&h, h.hf[f])[2])[2], HE(&h, HE(&h, HE(&h, h.hf[f])[2])[2])[2]};
    const int vq[4] = {HE(&h, e[0])[0], HE(&h, e[1])[0], HE(&h, e[2])[0], HE(&h, e[3])[0]};
    if (vV[vq[0]] != 3 || vV[vq[1]] != 3 || vV[vq[2]] != 3 || vV[vq[3]] != 3) continue;
    int fo[4], vo[4], boundary = 0;
    for (int r = 0; r < 4; r++) {
      const int twin = HE(&h, e[r])[3];
      if (twin == -1) { boundary = 1; break; }
      fo[r] = HE(&h, twin)[1];
      const int nx = HE(&h, HE(&h, twin)[2])[2];
      vo[r] = HE(&h, nx)[0];
    }
    if (boundary) continue;
    int nm = 0;
    for (int r = 0; r < 4; r++) if (non_manifold(&h, fo[r])) nm = 1;
    if (nm) continue;
    const int a = vV[vo[0]], b = vV[vo[1]], c = vV[vo[2]], d = vV[vo[3]];
    if ((a == 3 && b == 3) || (b == 3 && c == 3) || (c == 3 && d == 3) || (d == 3 && a == 3)) continue;
    if (a == 3 || b == 3 || c == 3 || d == 3) continue;
    if (a == 4 && b == 4 && c == 4 && d == 4) continue;
    for (int r = 0; r < 4; r++) { vm0[vq[r]] = 1; vm1[vq[r]] = vo[r]; vm2[vq[r]] = -1; }
    p[f] = 1;
    for (int r = 0; r < 4; r++) rf[fo[r]] = 1;
  }
  /* removeVertices3333 */
  size_t w = 0;
  for (int i = 0; i < nr_v; i++) {
    if (!vm0[i]) {
      vm2[i] = (int)w;
      for (int d = 0; d < 3; d++) { m->v.a[3 * w + d] = m->v.a[3 * (size_t)i + d]; m->n.a[3 * w + d] = m->n.a[3 * (size_t)i + d]; }
      w++;
    }
  }
  m->v.n = 3 * w; m->n.n = 3 * w;
  /* removeQuadrilaterals3333 */
  size_t wq = 0;
  int* nq = (int*)malloc(m->quads.n * sizeof(int) + 1);
  for (int f = 0; f < nr_q; f++) {
    if (rf[f]) continue;
    const int* q = m->quads.a + 4 * (size_t)f;
    for (int r = 0; r < 4; r++) nq[4 * wq + r] = p[f] ? vm2[vm1[q[r]]] : vm2[q[r]];
    wq++;
  }
  memcpy(m->quads.a, nq, 4 * wq * sizeof(int));
  m->quads.n = 4 * wq;
  free(nq); free(vV); free(p); free(rf); free(vm0); free(vm1); free(vm2);
  hmesh_free(&h);
}

/* minAngle (cpp_dmc/DualMarchingCubes.h:746-756): float side lengths, float acos */
static double min_angle(const double* v0, const double* v1, const double* v2) {
  const float a = sqrt((v0[0] - v1[0]) * (v0[0] - v1[0]) + (v0[1] - v1[1]) * (v0[1] - v1[1]) + (v0[2] - v1[2]) * (v0[2] - v1[2]));
  const float b = sqrt((v1[0] - v2[0]) * (v1[0] - v2[0]) + (v1[1] - v2[1]) * (v1[1] - v2[1]) + (v1[2] - v2[2]) * (v1[2] - v2[2]));
  const float c = sqrt((v2[0] - v0[0]) * (v2[0] - v0[0]) + (v2[1] - v0[1]) * (v2[1] - v0[1]) + (v2[2] - v0[2]) * (v2[2] - v0[2]));
  const float A = acosf((b * b + c * c - a * a) / (2 * b * c));
  const float B = acosf((a * a + c * c - b * b) / (2 * a * c));
  const float C = acosf((b * b + a * a - c * c) / (2 * b * a));
  const float mAB = (B < A) ? B : A;
  return (C < mAB) ? C : mAB;
}

/* collectTriangles (cpp_dmc/DualMarchingCubes.cpp:1387-1460) */
static void collect_triangles(const mesh_t* m, og_ivec* tris) {
  const size_t nr_q = m->quads.n / 4;
  const double* V = m->v.a;
  for (size_t i = 0; i < nr_q; i++) {
    const int v0 = m->quads.a[4 * i], v1 = m->quads.a[4 * i + 1], v2 = m->quads.a[4 * i + 2], v3 = m->quads.a[4 * i + 3];
    double a1 = min_angle(V + 3 * (size_t)v0, V + 3 * (size_t)v1, V + 3 * (size_t)v2);
    double a2 = min_angle(V + 3 * (size_t)v0, V + 3 * (size_t)v2, V + 3 * (size_t)v3);
    const double b1 = a2 < a1 ? a2 : a1, b2 = a1 < a2 ? a2 : a1;
    a1 = min_angle(V + 3 * (size_t)v1, V + 3 * (size_t)v3, V + 3 * (size_t)v0);
    a2 = min_angle(V + 3 * (size_t)v1, V + 3 * (size_t)v2, V + 3 * (size_t)v3);
    const double c1 = a2 < a1 ? a2 : a1, c2 = a1 < a2 ? a2 : a1;
    int t[6];
    if (b1 < c1 || (b1 == c1 && b2 <= c2)) { t[0] = v1; t[1] = v3; t[2] = v0; t[3] = v1; t[4] = v2; t[5] = v3; }
    else { t[0] = v0; t[1] = v1; t[2] = v2; t[3] = v0; t[4] = v2; t[5] = v3; }
    for (int r = 0; r < 6; r++) og_ivec_push(tris, t[r]);
  }
}

/* ---------------------------------------------------------------------------------------- */
/* exported entry points (ctypes)                                                             */
/* ---------------------------------------------------------------------------------------- */
static void fill_grid(og_grid* g, int nx, int ny, int nz, const double* origin, const double* spacing, const float* f) {
  g->nx = nx; g->ny = ny; g->nz = nz;
  for (int d = 0; d < 3; d++) { g->origin[d] = origin[d]; g->spacing[d] = spacing[d]; }
  g->f = f;
}

/* stage: 0 = full dualMC, 1 = front end only (quads + inherited colours + local coordinates) */
void* oracle_dmc_run(int nx, int ny, int nz, const double* origin, const double* spacing, const float* field,
                     double iso, int simplify, int flip, int stage) {
  og_grid g;
  fill_grid(&g, nx, ny, nz, origin, spacing, field);
  double* grad = estimate_gradient(&g, flip);
  mesh_t m;
  memset(&m, 0, sizeof m);
  dmc_result* r = (dmc_result*)calloc(1, sizeof(dmc_result));
  dmc_front(&g, grad, iso, &m, r->proj_fail);
  free(grad);
  if (stage == 1) {
    r->colors = (int*)malloc((m.colors.n + 1) * sizeof(int));
    memcpy(r->colors, m.colors.a, m.colors.n * sizeof(int));
    r->vcell = (int64_t*)malloc((m.vcell.n + 1) * sizeof(int64_t));
    memcpy(r->vcell, m.vcell.a, m.vcell.n * sizeof(int64_t));
    r->vuvw = (float*)malloc((m.vuvw.n + 1) * sizeof(float));
    memcpy(r->vuvw, m.vuvw.a, m.vuvw.n * sizeof(float));
  } else if (simplify) {
    simplify3x3y(&m);
    simplify3333(&m);
  }
  og_ivec tris = {0};
  hmesh h;
  memset(&h, 0, sizeof h);
  if (stage == 0) {
    halfedges((int)(m.v.n / 3), m.quads.a, (int)(m.quads.n / 4), &h);
    collect_triangles(&m, &tris);
  }
  r->nv = (int64_t)(m.v.n / 3);
  r->nq = (int64_t)(m.quads.n / 4);
  r->nt = (int64_t)(tris.n / 3);
  r->nhe = stage == 0 ? 4 * r->nq : 0;
  r->v = m.v.a; r->n = m.n.a; r->quads = m.quads.a; r->tris = tris.a;
  r->he = h.he; r->he_v = h.hv; r->he_f = h.hf;
  og_ivec_free(&m.colors); og_lvec_free(&m.vcell); og_fvec_free(&m.vuvw);
  return r;
}

void oracle_dmc_sizes(void* hd, int64_t* out4) {
  dmc_result* r = (dmc_result*)hd;
  out4[0] = r->nv; out4[1] = r->nq; out4[2] = r->nt; out4[3] = r->nhe;
}

void oracle_dmc_copy(void* hd, double* v, double* n, int* quads, int* tris, int* he, int* he_v, int* he_f) {
  dmc_result* r = (dmc_result*)hd;
  if (v && r->nv) memcpy(v, r->v, 3 * r->nv * sizeof(double));
  if (n && r->nv) memcpy(n, r->n, 3 * r->nv * sizeof(double));
  if (quads && r->nq) memcpy(quads, r->quads, 4 * r->nq * sizeof(int));
  if (tris && r->nt) memcpy(tris, r->tris, 3 * r->nt * sizeof(int));
  if (he && r->nhe) memcpy(he, r->he, 5 * r->nhe * sizeof(int));
  if (he_v && r->he_v && r->nv) memcpy(he_v, r->he_v, r->nv * sizeof(int));
  if (he_f && r->he_f && r->nq) memcpy(he_f, r->he_f, r->nq * sizeof(int));
}

void oracle_dmc_copy_front(void* hd, int* colors, int64_t* vcell, float* vuvw) {
  dmc_result* r = (dmc_result*)hd;
  if (colors && r->colors) memcpy(colors, r->colors, r->nq * sizeof(int));
  if (vcell && r->vcell) memcpy(vcell, r->vcell, r->nv * sizeof(int64_t));
  if (vuvw && r->vuvw) memcpy(vuvw, r->vuvw, 3 * r->nv * sizeof(float));
}

void oracle_dmc_proj_fail(void* hd, int64_t* out2) {
  dmc_result* r = (dmc_result*)hd;
  out2[0] = r->proj_fail[0]; out2[1] = r->proj_fail[1];
}

void oracle_dmc_free(void* hd) {
  dmc_result* r = (dmc_result*)hd;
  free(r->v); free(r->n); free(r->quads); free(r->tris); free(r->he); free(r->he_v); free(r->he_f);
  free(r->colors); free(r->vcell); free(r->vuvw);
  free(r);
}

/* colour + valence stage on a given quad mesh (for per-stage checks) */
void oracle_dmc_color_valence(int nr_v, int nr_q, const int* quads, int* colors_inout, int* valence_out) {
  hmesh h;
  halfedges(nr_v, quads, nr_q, &h);
  color_faces_full(&h, colors_inout);
  int* vV = vertex_valence(&h);
  memcpy(valence_out, vV, (size_t)nr_v * sizeof(int));
  free(vV);
  hmesh_free(&h);
}

/* Halfedges of a triangle (P = 3) or quad (P = 4) mesh with the rules of halfedges()
 * (cpp_dmc/DualMarchingCubes.cpp:488-671); used as the oracle of the TMC halfedge output, whose
 * reference kernel (cuda_tmc/MarchingCubes.cu:2284-2336) registers only the first edge of each
 * triangle. he5: 5 ints per halfedge. */
int64_t oracle_halfedges(const int* faces, int P, int nr_f, int nr_v, int* he5, int* hv, int* hf) {
  hmesh h;
  halfedges_p(nr_v, faces, P, nr_f, &h);
  memcpy(he5, h.he, (size_t)5 * P * nr_f * sizeof(int));
  memcpy(hv, h.hv, (size_t)nr_v * sizeof(int));
  memcpy(hf, h.hf, (size_t)nr_f * sizeof(int));
  int64_t nm = 0;
  for (int64_t e = 0; e < (int64_t)P * nr_f; e++) nm += h.he[5 * e + 4] != 0;
  hmesh_free(&h);
  return nm;
}
