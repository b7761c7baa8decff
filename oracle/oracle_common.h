/* Shared pieces of the CPU oracle (test infrastructure only; never part of the product path).
 *
 * The oracle restates the reference's single-threaded CPU algorithms in plain C:
 *   dmc_oracle.c  - cpp_dmc/DualMarchingCubes.cpp (dualMC and its mesh post-processing)
 *   tmc_oracle.c  - mc/MarchingCubes.cpp (t_mc and p_slice)
 * Every function cites the reference lines it follows.  The oracle is pinned against the
 * reference compiled from its own sources (oracle/_ref, built by `make -C oracle ref`) and
 * against the golden fixtures in tests/golden/.
 */
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../tmc_gb300/csrc/mc_tables.h"

/* ---------------------------------------------------------------------------------------- */
/* growable arrays                                                                          */
/* ---------------------------------------------------------------------------------------- */
#define OG_VEC(name, T)                                                                        \
  typedef struct { T* a; size_t n, cap; } name;                                              \
  static inline void name##_push(name* v, T x) {                                             \
    if (v->n == v->cap) {                                                                    \
      v->cap = v->cap ? 2 * v->cap : 64;                                                     \
      v->a = (T*)realloc(v->a, v->cap * sizeof(T));                                          \
    }                                                                                        \
    v->a[v->n++] = x;                                                                        \
  }                                                                                          \
  static inline void name##_free(name* v) { free(v->a); v->a = NULL; v->n = v->cap = 0; }

OG_VEC(og_ivec, int)
OG_VEC(og_dvec, double)
OG_VEC(og_fvec, float)
OG_VEC(og_lvec, int64_t)

/* ---------------------------------------------------------------------------------------- */
/* grid                                                                                     */
/* ---------------------------------------------------------------------------------------- */
typedef struct {
  int nx, ny, nz;
  double origin[3];
  double spacing[3];
  const float* f; /* x fastest */
} og_grid;

/* UniformGrid::global_index (cpp_dmc/UniformGrid.h:267, mc/MarchingCubes.h:218), int arithmetic
 * as in the reference (wraps under -fwrapv beyond 2^31 points). */
static inline int og_gindex(const og_grid* g, int i, int j, int k) { return k * g->ny * g->nx + j * g->nx + i; }
static inline double og_s(const og_grid* g, int i, int j, int k) {
  return (double)g->f[((size_t)k * g->ny + j) * g->nx + i];
}

/* ---------------------------------------------------------------------------------------- */
/* cell topology (vertex v = (v&1, (v>>1)&1, (v>>2)&1))                                     */
/* ---------------------------------------------------------------------------------------- */
/* edge end vertices: l_edges_ in cpp_dmc/DualMarchingCubes.cpp:109, mc/MarchingCubes.cpp:331 */
static const int OG_EDGE_V[12][2] = {{0, 1}, {1, 3}, {2, 3}, {0, 2}, {4, 5}, {5, 7},
                                     {6, 7}, {4, 6}, {0, 4}, {1, 5}, {3, 7}, {2, 6}};
/* oriented faces seen from outside: v_face_/e_face_ (cpp_dmc/DualMarchingCubes.h:286-288) */
static const int OG_FACE_V[6][4] = {{0, 2, 1, 3}, {5, 7, 4, 6}, {4, 0, 5, 1}, {2, 6, 3, 7}, {4, 6, 0, 2}, {1, 3, 5, 7}};
static const int OG_FACE_E[6][4] = {{3, 2, 1, 0}, {5, 6, 7, 4}, {8, 0, 9, 4}, {11, 6, 10, 2}, {7, 11, 3, 8}, {1, 10, 5, 9}};
/* global edge of local edge e: grid point offset and axis; gei_pattern_
 * (cpp_dmc/DualMarchingCubes.h:212, mc/MarchingCubes.cpp:327) */
static const int OG_EDGE_GLOBAL[12][4] = {{0, 0, 0, 0}, {1, 0, 0, 1}, {0, 1, 0, 0}, {0, 0, 0, 1},
                                          {0, 0, 1, 0}, {1, 0, 1, 1}, {0, 1, 1, 0}, {0, 0, 1, 1},
                                          {0, 0, 0, 2}, {1, 0, 0, 2}, {1, 1, 0, 2}, {0, 1, 0, 2}};
/* quad slot of a cell's vertex around a dual edge, by the side of the edge's first end vertex;
 * e_talbe in get_vertex_pos (cpp_dmc/DualMarchingCubes.h:223) */
static const int OG_QUAD_SLOT[12][2] = {{0, 0}, {0, 0}, {3, 1}, {3, 1}, {1, 3}, {1, 3},
                                        {2, 2}, {2, 2}, {0, 0}, {3, 1}, {2, 2}, {1, 3}};
/* direction / constant of the local coordinates of an edge point; e_ and c_ constants in
 * getLocalCoordinates (cpp_dmc/DualMarchingCubes.h:396-397) */
static const int OG_EDGE_DIR[12][3] = {{1, 0, 0}, {0, 1, 0}, {1, 0, 0}, {0, 1, 0}, {1, 0, 0}, {0, 1, 0},
                                       {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, 1}, {0, 0, 1}, {0, 0, 1}};
static const int OG_EDGE_CON[12][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {1, 0, 1},
                                       {0, 1, 1}, {0, 0, 1}, {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}};

static inline int og_is_ambiguous(unsigned c) { return (int)((TMC_AMBIGUOUS[c >> 6] >> (c & 63)) & 1u); }
static inline int og_contour_start(unsigned c) { return (TMC_CONTOUR_START[c >> 1] >> (4 * (c & 1))) & 0xF; }

/* contours of the MC polygon: up to 4 closed loops, 12 edges in total */
typedef struct {
  int n;
  int size[4];
  int e[4][12];
} og_contours;

/* Connect oriented face segments (to[e] = next edge, -1 unset) into closed contours, starting
 * each at its lowest edge: the connect loop of mc_polygon (cpp_dmc/DualMarchingCubes.cpp:443-463)
 * and p_slice (mc/MarchingCubes.cpp:690-709). */
static inline void og_connect(const int to_in[12], og_contours* c) {
  int to[12], set[12];
  for (int e = 0; e < 12; e++) { to[e] = to_in[e]; set[e] = 0; }
  for (int e = 0; e < 12; e++) if (to[e] >= 0) { set[e] = 1; set[to[e]] = 1; }
  c->n = 0;
  for (int e = 0; e < 12; e++) {
    if (!set[e]) continue;
    int t = c->n, pos = 0, nxt = to[e];
    c->e[t][pos] = e;
    while (nxt != e) {
      pos++;
      c->e[t][pos] = nxt;
      int in = nxt;
      nxt = to[in];
      set[in] = 0;
    }
    c->size[t] = pos + 1;
    c->n++;
  }
}

/* Face-segment rules for the 14 face cases (f_case bit b set when face vertex b is >= iso);
 * cases 6 and 9 need the decider: `sep` selects the branch the reference takes when the
 * asymptotic decider value is >= (DMC) or > (TMC) the isovalue.  Follows the switch in
 * cpp_dmc/DualMarchingCubes.cpp:357-425 (identical rules in mc/MarchingCubes.cpp:495-668). */
static inline void og_face_rule(int fc, int sep, const int fe[4], int to[12]) {
  switch (fc) {
    case 1: to[fe[0]] = fe[3]; break;
    case 2: to[fe[1]] = fe[0]; break;
    case 3: to[fe[1]] = fe[3]; break;
    case 4: to[fe[3]] = fe[2]; break;
    case 5: to[fe[0]] = fe[2]; break;
    case 6:
      if (sep) { to[fe[3]] = fe[0]; to[fe[1]] = fe[2]; }
      else { to[fe[1]] = fe[0]; to[fe[3]] = fe[2]; }
      break;
    case 7: to[fe[1]] = fe[2]; break;
    case 8: to[fe[2]] = fe[1]; break;
    case 9:
      if (sep) { to[fe[0]] = fe[1]; to[fe[2]] = fe[3]; }
      else { to[fe[0]] = fe[3]; to[fe[2]] = fe[1]; }
      break;
    case 10: to[fe[2]] = fe[0]; break;
    case 11: to[fe[2]] = fe[3]; break;
    case 12: to[fe[3]] = fe[1]; break;
    case 13: to[fe[0]] = fe[1]; break;
    case 14: to[fe[3]] = fe[0]; break;
    default: break;
  }
}

static inline int og_face_case(unsigned cs, int f) {
  return (int)(((cs >> OG_FACE_V[f][0]) & 1) | ((cs >> OG_FACE_V[f][1]) & 1) << 1 |
               ((cs >> OG_FACE_V[f][2]) & 1) << 2 | ((cs >> OG_FACE_V[f][3]) & 1) << 3);
}

/* asymptotic decider (cpp_dmc/DualMarchingCubes.h:330, mc/MarchingCubes.cpp:487) */
static inline double og_decider(double f0, double f1, double f2, double f3) {
  return (f0 * f3 - f1 * f2) / (f0 + f3 - f1 - f2);
}

/* The contour of an unambiguous case: the face rules (no decider needed) connected, then
 * rotated to the start edge the reference's table uses (cpp_dmc/LookupTables.h r_pattern,
 * read by mc_polygon(i_case), cpp_dmc/DualMarchingCubes.cpp:470-487). */
static inline void og_table_contour(unsigned cs, og_contours* c) {
  int to[12];
  for (int e = 0; e < 12; e++) to[e] = -1;
  for (int f = 0; f < 6; f++) og_face_rule(og_face_case(cs, f), 0, OG_FACE_E[f], to);
  og_connect(to, c);
  if (c->n == 1) {
    int s = og_contour_start(cs), sz = c->size[0], r = 0;
    for (int p = 0; p < sz; p++) if (c->e[0][p] == s) r = p;
    int tmp[12];
    for (int p = 0; p < sz; p++) tmp[p] = c->e[0][(p + r) % sz];
    for (int p = 0; p < sz; p++) c->e[0][p] = tmp[p];
  }
}

/* unpack triangle t (0..4) of an unambiguous case: t_pattern (mc/MarchingCubes.h:471) */
static inline int og_tri_count(unsigned cs) { return (int)(TMC_TRIANGLES[cs] & 0xF); }
static inline int og_tri_edge(unsigned cs, int t, int k) { return (int)((TMC_TRIANGLES[cs] >> (4 + 4 * (3 * t + k))) & 0xF); }
