/*
 * nmag_oracle.c -- CPU restatement (test infrastructure only) of nsim's
 * micromagnetic right-hand side: P1 tetrahedral discretisation, FEM/BEM
 * (Fredkin-Koehler) demagnetisation with Lindholm double-layer weights,
 * exchange, uniaxial anisotropy, Zeeman and the LLG equation.
 *
 * It supplies the expected results of the CUDA library's parity tests and the
 * CPU baseline of bench.py, never part of the product.  Parity with the reference is UNPINNED (the
 * reference cannot run here and ships no golden vectors); see the header.
 *
 * Floating-point contract: compiled with -ffp-contract=off so the per-tet
 * geometry and assembly below are evaluated in exactly the written order; the
 * device assembly kernels follow the same operation order (and are built with
 * --fmad=false), which makes CSR values bit-identical between the two.
 */
#include "nmag_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OM_PI 3.141592653589793 /* OCaml's pi = 4 atan 1 */

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* ---------------------------------------------------------------- geometry */

/* Barycentric gradients of a tetrahedron: rows of the inverse point matrix
 * (Simplex.get_inv_point_matrices; used by fem.ml:1603-1641 for every
 * integral and by bem3d.ml:45-50 as face equations). */
static void tet_geometry(const double *p0, const double *p1, const double *p2, const double *p3,
                         double dL[4][3], double *adet) {
  double e1[3], e2[3], e3[3], c23[3], c31[3], c12[3];
  for (int d = 0; d < 3; ++d) { e1[d] = p1[d] - p0[d]; e2[d] = p2[d] - p0[d]; e3[d] = p3[d] - p0[d]; }
  c23[0] = e2[1] * e3[2] - e2[2] * e3[1]; c23[1] = e2[2] * e3[0] - e2[0] * e3[2]; c23[2] = e2[0] * e3[1] - e2[1] * e3[0];
  c31[0] = e3[1] * e1[2] - e3[2] * e1[1]; c31[1] = e3[2] * e1[0] - e3[0] * e1[2]; c31[2] = e3[0] * e1[1] - e3[1] * e1[0];
  c12[0] = e1[1] * e2[2] - e1[2] * e2[1]; c12[1] = e1[2] * e2[0] - e1[0] * e2[2]; c12[2] = e1[0] * e2[1] - e1[1] * e2[0];
  double det = e1[0] * c23[0] + e1[1] * c23[1] + e1[2] * c23[2];
  double inv = 1.0 / det;
  for (int d = 0; d < 3; ++d) {
    dL[1][d] = c23[d] * inv; dL[2][d] = c31[d] * inv; dL[3][d] = c12[d] * inv;
    dL[0][d] = -((dL[1][d] + dL[2][d]) + dL[3][d]);
  }
  *adet = fabs(det);
}

/* snippets.ml:1229-1258 triangle_space_angle_3d: solid angle of triangle
 * (p0,p1,p2) seen from obs (van Oosterom-Strackee form). */
double om_triangle_space_angle(const double *obs, const double *p0, const double *p1, const double *p2) {
  double r0[3], r1[3], r2[3];
  for (int i = 0; i < 3; ++i) { r0[i] = p0[i] - obs[i]; r1[i] = p1[i] - obs[i]; r2[i] = p2[i] - obs[i]; }
  double r0l = sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
  double r1l = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  double r2l = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  double sp01 = r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2];
  double sp12 = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
  double sp20 = r2[0] * r0[0] + r2[1] * r0[1] + r2[2] * r0[2];
  double num = r0l * r1l * r2l + r0l * sp12 + r1l * sp20 + r2l * sp01;
  double den = sqrt(2.0 * (r1l * r2l + sp12) * (r2l * r0l + sp20) * (r0l * r1l + sp01));
  if (den == 0.0) return 0.0;
  double q = num / den;
  if (q < -1.0) q = -1.0; else if (q > 1.0) q = 1.0;
  return 2.0 * acos(q);
}

static int cmp_i32(const void *a, const void *b) {
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

static int row_find(const int32_t *cols, int lo, int hi, int32_t c) {
  while (lo < hi) { int mid = (lo + hi) >> 1; if (cols[mid] < c) lo = mid + 1; else hi = mid; }
  return lo;
}

/* ---------------------------------------------------------------- build */

int om_build(om_mesh *M, int N, const double *coords, int T, const int32_t *tets) {
  memset(M, 0, sizeof(*M));
  if (N <= 0 || T <= 0) return -1;
  M->n_nodes = N; M->n_tets = T;
  M->coords = malloc(sizeof(double) * 3 * N); memcpy(M->coords, coords, sizeof(double) * 3 * N);
  M->tets = malloc(sizeof(int32_t) * 4 * T); memcpy(M->tets, tets, sizeof(int32_t) * 4 * T);
  for (int i = 0; i < 4 * T; ++i) if (tets[i] < 0 || tets[i] >= N) return -2;

  /* node -> tet adjacency, ascending tet order */
  M->nt_ptr = xcalloc(N + 1, sizeof(int32_t));
  for (int i = 0; i < 4 * T; ++i) M->nt_ptr[tets[i] + 1]++;
  for (int i = 0; i < N; ++i) M->nt_ptr[i + 1] += M->nt_ptr[i];
  M->nt_idx = xcalloc(4 * T, sizeof(int32_t));
  int32_t *fill = xcalloc(N, sizeof(int32_t));
  for (int t = 0; t < T; ++t)
    for (int a = 0; a < 4; ++a) { int v = tets[4 * t + a]; M->nt_idx[M->nt_ptr[v] + fill[v]++] = t; }
  free(fill);

  /* per-tet geometry */
  M->dL = xcalloc(12 * (size_t)T, sizeof(double)); M->adet = xcalloc(T, sizeof(double));
  for (int t = 0; t < T; ++t) {
    const int32_t *v = tets + 4 * t;
    tet_geometry(coords + 3 * v[0], coords + 3 * v[1], coords + 3 * v[2], coords + 3 * v[3],
                 (double(*)[3])(M->dL + 12 * (size_t)t), M->adet + t);
    if (!(M->adet[t] > 0.0)) return -3; /* degenerate tet */
  }

  /* face neighbours (fem.ml:2785-2818 uses sx.ms_neighbours; outer face = no neighbour) */
  M->nbr = xcalloc(4 * (size_t)T, sizeof(int32_t));
  for (int t = 0; t < T; ++t) {
    const int32_t *v = tets + 4 * t;
    for (int f = 0; f < 4; ++f) {
      int32_t fv[3], k = 0;
      for (int a = 0; a < 4; ++a) if (a != f) fv[k++] = v[a];
      int32_t vmin = fv[0] < fv[1] ? (fv[0] < fv[2] ? fv[0] : fv[2]) : (fv[1] < fv[2] ? fv[1] : fv[2]);
      int32_t found = -1;
      for (int q = M->nt_ptr[vmin]; q < M->nt_ptr[vmin + 1]; ++q) {
        int u = M->nt_idx[q]; if (u == t) continue;
        const int32_t *w = tets + 4 * u; int hit = 0;
        for (int b = 0; b < 4; ++b) hit += (w[b] == fv[0]) + (w[b] == fv[1]) + (w[b] == fv[2]);
        if (hit == 3) { found = u; break; }
      }
      M->nbr[4 * t + f] = found;
    }
  }

  /* boundary nodes ("phi[outer]"): nodes on an outer face; short index ascending
     in node (= DOF) order (fem.ml:711-756 orders restricted vectors by DOF). */
  M->b_of_node = xcalloc(N, sizeof(int32_t));
  for (int t = 0; t < T; ++t)
    for (int f = 0; f < 4; ++f) if (M->nbr[4 * t + f] < 0)
      for (int a = 0; a < 4; ++a) if (a != f) M->b_of_node[tets[4 * t + a]] = 1;
  int nb = 0;
  for (int i = 0; i < N; ++i) { if (M->b_of_node[i]) M->b_of_node[i] = nb++; else M->b_of_node[i] = -1; }
  M->nb = nb;
  M->node_of_b = xcalloc(nb, sizeof(int32_t));
  for (int i = 0; i < N; ++i) if (M->b_of_node[i] >= 0) M->node_of_b[M->b_of_node[i]] = i;

  /* CSR pattern: every node pair sharing a tet (PETSc AIJ keeps each
     position MatSetValues touched, nsim.ml:1758 + fem.ml:5107-5150). */
  M->row_ptr = xcalloc(N + 1, sizeof(int32_t));
  int32_t *buf = xcalloc(4 * 64, sizeof(int32_t));
  int bufcap = 256;
  int32_t *cols_tmp = NULL; size_t cols_cap = 0, cols_len = 0;
  for (int i = 0; i < N; ++i) {
    int deg = M->nt_ptr[i + 1] - M->nt_ptr[i];
    if (4 * deg > bufcap) { bufcap = 4 * deg; buf = realloc(buf, sizeof(int32_t) * bufcap); }
    int n = 0;
    for (int q = M->nt_ptr[i]; q < M->nt_ptr[i + 1]; ++q)
      for (int a = 0; a < 4; ++a) buf[n++] = tets[4 * M->nt_idx[q] + a];
    qsort(buf, n, sizeof(int32_t), cmp_i32);
    int u = 0;
    for (int k = 0; k < n; ++k) if (u == 0 || buf[k] != buf[u - 1]) buf[u++] = buf[k];
    if (cols_len + u > cols_cap) { cols_cap = 2 * (cols_len + u) + 1024; cols_tmp = realloc(cols_tmp, sizeof(int32_t) * cols_cap); }
    memcpy(cols_tmp + cols_len, buf, sizeof(int32_t) * u); cols_len += u;
    M->row_ptr[i + 1] = (int32_t)cols_len;
  }
  free(buf);
  M->nnz = (int)cols_len; M->col_idx = cols_tmp;
  size_t nnz = cols_len;
  M->K = xcalloc(nnz, sizeof(double));
  for (int d = 0; d < 3; ++d) { M->G[d] = xcalloc(nnz, sizeof(double)); M->D[d] = xcalloc(nnz, sizeof(double)); }
  M->vol = xcalloc(N, sizeof(double));

  /* Values.  Per row, tets ascending, local columns b = 0..3:
       K  += (|det|/6)  dL_a . dL_b                (<d/dxj a || d/dxj b>)
       G_d += (|det|/24) dL_b[d]                   (<a || d/dxj b>)
     outer-surface part of <rho || D/Dxj m(j)> (fem.ml:5124-5150), face f outer, a,b != f:
       S_d += (1 + delta_ab) (|det|/24) dL_f[d]     (= -int_face phi_a phi_b n_d)
     volumes (fem.ml:1757-1790): V_i += |det|/24.                                */
  double *S[3];
  for (int d = 0; d < 3; ++d) S[d] = xcalloc(nnz, sizeof(double));
  for (int i = 0; i < N; ++i) {
    int lo = M->row_ptr[i], hi = M->row_ptr[i + 1];
    for (int q = M->nt_ptr[i]; q < M->nt_ptr[i + 1]; ++q) {
      int t = M->nt_idx[q];
      const int32_t *v = tets + 4 * t;
      const double(*dL)[3] = (const double(*)[3])(M->dL + 12 * (size_t)t);
      double ad = M->adet[t];
      int a = 0; while (v[a] != i) ++a;
      double kc = ad / 6.0, gc = ad / 24.0;
      for (int b = 0; b < 4; ++b) {
        int pos = row_find(M->col_idx, lo, hi, v[b]);
        M->K[pos] += kc * ((dL[a][0] * dL[b][0] + dL[a][1] * dL[b][1]) + dL[a][2] * dL[b][2]);
        for (int d = 0; d < 3; ++d) M->G[d][pos] += gc * dL[b][d];
      }
      M->vol[i] += gc;
    }
    for (int q = M->nt_ptr[i]; q < M->nt_ptr[i + 1]; ++q) {
      int t = M->nt_idx[q];
      const int32_t *v = tets + 4 * t;
      const double(*dL)[3] = (const double(*)[3])(M->dL + 12 * (size_t)t);
      int a = 0; while (v[a] != i) ++a;
      for (int f = 0; f < 4; ++f) {
        if (f == a || M->nbr[4 * t + f] >= 0) continue;
        double sf[3];
        for (int d = 0; d < 3; ++d) sf[d] = (M->adet[t] / 24.0) * dL[f][d];
        for (int b = 0; b < 4; ++b) {
          if (b == f) continue;
          int pos = row_find(M->col_idx, lo, hi, v[b]);
          for (int d = 0; d < 3; ++d) S[d][pos] += (a == b) ? (sf[d] + sf[d]) : sf[d];
        }
      }
    }
  }
  for (int d = 0; d < 3; ++d) {
    for (size_t k = 0; k < nnz; ++k) M->D[d][k] = M->G[d][k] + S[d][k];
    free(S[d]);
  }

  /* Surface triangles, reference rule (bem3d.ml:83-176): for each boundary
     node in short order, each tet containing it (ascending), each opposing
     vertex: emit the face if all its vertices are boundary nodes whose short
     index is >= this node's.  The list is built by prepending, so the final
     order is the reverse of discovery.  Outward normal = -dL_f/|dL_f|. */
  int cap = 1024, cnt = 0;
  int32_t *tri_tmp = malloc(sizeof(int32_t) * 3 * cap);
  double *nrm_tmp = malloc(sizeof(double) * 3 * cap);
  for (int sb = 0; sb < nb; ++sb) {
    int node = M->node_of_b[sb];
    for (int q = M->nt_ptr[node]; q < M->nt_ptr[node + 1]; ++q) {
      int t = M->nt_idx[q];
      const int32_t *v = tets + 4 * t;
      int bidx[4], a = -1;
      for (int k = 0; k < 4; ++k) { bidx[k] = M->b_of_node[v[k]]; if (bidx[k] == sb) a = k; }
      for (int op = 0; op < 4; ++op) {
        if (op == a) continue;
        int ok = 1;
        for (int k = 0; k < 4 && ok; ++k) {
          if (k == op) continue;
          if (bidx[k] < bidx[a]) ok = 0; else if (bidx[k] == -1) ok = 0;
        }
        if (!ok) continue;
        if (cnt == cap) { cap *= 2; tri_tmp = realloc(tri_tmp, sizeof(int32_t) * 3 * cap); nrm_tmp = realloc(nrm_tmp, sizeof(double) * 3 * cap); }
        int k3 = 0;
        for (int k = 0; k < 4; ++k) if (k != op) tri_tmp[3 * cnt + k3++] = bidx[k];
        const double *g = M->dL + 12 * (size_t)t + 3 * op;
        double r = -1.0 / sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        for (int d = 0; d < 3; ++d) nrm_tmp[3 * cnt + d] = r * g[d];
        ++cnt;
      }
    }
  }
  M->ntri = cnt;
  M->tri = xcalloc(3 * (size_t)cnt, sizeof(int32_t)); M->tri_normal = xcalloc(3 * (size_t)cnt, sizeof(double));
  for (int k = 0; k < cnt; ++k) {
    memcpy(M->tri + 3 * k, tri_tmp + 3 * (cnt - 1 - k), 3 * sizeof(int32_t));
    memcpy(M->tri_normal + 3 * k, nrm_tmp + 3 * (cnt - 1 - k), 3 * sizeof(double));
  }
  free(tri_tmp); free(nrm_tmp);

  /* interior solid angles (mesh.ml:1792-1821), tets ascending */
  M->solid_angle = xcalloc(nb, sizeof(double));
  for (int sb = 0; sb < nb; ++sb) {
    int node = M->node_of_b[sb];
    double acc = 0.0;
    for (int q = M->nt_ptr[node]; q < M->nt_ptr[node + 1]; ++q) {
      const int32_t *v = tets + 4 * M->nt_idx[q];
      int ix0 = 0; while (v[ix0] != node) ++ix0;
      int ix1 = ix0 <= 0 ? 1 : 0, ix2 = ix0 <= 1 ? 2 : 1, ix3 = ix0 <= 2 ? 3 : 2;
      acc += fabs(om_triangle_space_angle(coords + 3 * v[ix0], coords + 3 * v[ix1], coords + 3 * v[ix2], coords + 3 * v[ix3]));
    }
    M->solid_angle[sb] = acc;
  }
  return 0;
}

/* ---------------------------------------------------------------- BEM fill */

typedef struct { double p[3][3], s_l[3], eta[3][3], zeta_v[3], gam[3][3], factor, maxgeo; int ok; } om_tri_geo;

/* Per-triangle setup of the Lindholm block routine (bem3d_stubs.c:466-525). */
static void tri_setup(const om_mesh *M, int t, om_tri_geo *g) {
  const int32_t *tv = M->tri + 3 * t;
  double s[3][3], xi[3][3];
  g->ok = 0; g->maxgeo = 0.0;
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) {
      g->p[k][d] = M->coords[3 * M->node_of_b[tv[k]] + d];
      double ax = fabs(g->p[k][d]); if (ax > g->maxgeo) g->maxgeo = ax;
    }
  for (int d = 0; d < 3; ++d) { s[0][d] = g->p[2][d] - g->p[1][d]; s[1][d] = g->p[0][d] - g->p[2][d]; s[2][d] = g->p[1][d] - g->p[0][d]; }
  for (int k = 0; k < 3; ++k) {
    g->s_l[k] = sqrt(s[k][0] * s[k][0] + s[k][1] * s[k][1] + s[k][2] * s[k][2]);
    if (g->s_l[k] == 0.0) return;
    double inv = 1.0 / g->s_l[k];
    for (int d = 0; d < 3; ++d) xi[k][d] = s[k][d] * inv;
  }
  double z[3];
  z[0] = s[1][1] * s[2][2] - s[1][2] * s[2][1]; z[1] = s[1][2] * s[2][0] - s[1][0] * s[2][2]; z[2] = s[1][0] * s[2][1] - s[1][1] * s[2][0];
  double len = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  if (len == 0.0) return;
  double area = 0.5 * len, inv = 1.0 / len;
  for (int d = 0; d < 3; ++d) g->zeta_v[d] = z[d] * inv;
  double c01 = xi[0][0] * xi[1][0] + xi[0][1] * xi[1][1] + xi[0][2] * xi[1][2];
  double c12 = xi[1][0] * xi[2][0] + xi[1][1] * xi[2][1] + xi[1][2] * xi[2][2];
  double c20 = xi[2][0] * xi[0][0] + xi[2][1] * xi[0][1] + xi[2][2] * xi[0][2];
  for (int k = 0; k < 3; ++k) {
    const double *zv = g->zeta_v;
    g->eta[k][0] = zv[1] * xi[k][2] - zv[2] * xi[k][1];
    g->eta[k][1] = zv[2] * xi[k][0] - zv[0] * xi[k][2];
    g->eta[k][2] = zv[0] * xi[k][1] - zv[1] * xi[k][0];
  }
  g->gam[0][0] = 1.0; g->gam[0][1] = c01; g->gam[0][2] = c20;
  g->gam[1][0] = c01; g->gam[1][1] = 1.0; g->gam[1][2] = c12;
  g->gam[2][0] = c20; g->gam[2][1] = c12; g->gam[2][2] = 1.0;
  double f = 1.0 * (1.0 / (8.0 * OM_PI * area));
  const double *n = M->tri_normal + 3 * t;
  if (g->zeta_v[0] * n[0] + g->zeta_v[1] * n[1] + g->zeta_v[2] * n[2] < 0.0) f = -f;
  g->factor = f;
  g->ok = 1;
}

/* One observer / triangle pair (bem3d_stubs.c:527-604).  geo_eps follows the
 * reference's running maximum over the triangle and the observers visited so
 * far in the same row sweep. */
static void lindholm(const om_tri_geo *g, const double *obs, double geo_eps, double lh[3]) {
  double r[3][3], rl[3];
  lh[0] = lh[1] = lh[2] = 0.0;
  for (int k = 0; k < 3; ++k) {
    for (int d = 0; d < 3; ++d) r[k][d] = g->p[k][d] - obs[d];
    rl[k] = sqrt(r[k][0] * r[k][0] + r[k][1] * r[k][1] + r[k][2] * r[k][2]);
  }
  if (rl[0] <= 0.0 || rl[1] <= 0.0 || rl[2] <= 0.0) return;
  double vlog[3];
  vlog[0] = log((rl[1] + rl[2] + g->s_l[0]) / (rl[1] + rl[2] - g->s_l[0]));
  vlog[1] = log((rl[2] + rl[0] + g->s_l[1]) / (rl[2] + rl[0] - g->s_l[1]));
  vlog[2] = log((rl[0] + rl[1] + g->s_l[2]) / (rl[0] + rl[1] - g->s_l[2]));
  double sp01 = r[0][0] * r[1][0] + r[0][1] * r[1][1] + r[0][2] * r[1][2];
  double sp12 = r[1][0] * r[2][0] + r[1][1] * r[2][1] + r[1][2] * r[2][2];
  double sp20 = r[2][0] * r[0][0] + r[2][1] * r[0][1] + r[2][2] * r[0][2];
  double num = rl[0] * rl[1] * rl[2] + rl[0] * sp12 + rl[1] * sp20 + rl[2] * sp01;
  double den = sqrt(2.0 * (rl[1] * rl[2] + sp12) * (rl[2] * rl[0] + sp20) * (rl[0] * rl[1] + sp01));
  if (den == 0.0) return;
  double angle = num / den;
  if (angle < -1.0) angle = -1.0; else if (angle > 1.0) angle = 1.0;
  angle = 2.0 * acos(angle);
  double zeta = g->zeta_v[0] * r[0][0] + g->zeta_v[1] * r[0][1] + g->zeta_v[2] * r[0][2];
  if (zeta < 0.0) angle = -angle;
  double f = g->factor;
  if (fabs(zeta) < geo_eps) f = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double *rn = r[(k + 1) % 3];
    double e = g->eta[k][0] * rn[0] + g->eta[k][1] * rn[1] + g->eta[k][2] * rn[2];
    double gl = g->gam[k][0] * vlog[0] + g->gam[k][1] * vlog[1] + g->gam[k][2] * vlog[2];
    lh[k] = f * g->s_l[k] * (angle * e - zeta * gl);
  }
}

int om_fill_bem(om_mesh *M, int nthreads) {
  int nb = M->nb, nt = M->ntri;
  free(M->bem);
  M->bem = xcalloc((size_t)nb * nb, sizeof(double));
  if (!M->bem) return -1;
  om_tri_geo *geo = xcalloc(nt, sizeof(om_tri_geo));
  for (int t = 0; t < nt; ++t) tri_setup(M, t, &geo[t]);
  double *obs_max = xcalloc(nb, sizeof(double));
  double run = 0.0;
  for (int k = 0; k < nb; ++k) {
    const double *o = M->coords + 3 * M->node_of_b[k];
    for (int d = 0; d < 3; ++d) if (fabs(o[d]) > run) run = fabs(o[d]);
    obs_max[k] = run;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (int k = 0; k < nb; ++k) {
    double *row = M->bem + (size_t)k * nb;
    const double *obs = M->coords + 3 * M->node_of_b[k];
    for (int t = 0; t < nt; ++t) {
      const om_tri_geo *g = &geo[t];
      if (!g->ok) continue;
      double mg = g->maxgeo > obs_max[k] ? g->maxgeo : obs_max[k];
      double lh[3];
      lindholm(g, obs, mg * 1e-13, lh);
      const int32_t *tv = M->tri + 3 * t;
      row[tv[0]] += lh[0]; row[tv[1]] += lh[1]; row[tv[2]] += lh[2];
    }
    row[k] += M->solid_angle[k] / (4.0 * OM_PI) - 1.0;
  }
  free(geo); free(obs_max);
  return 0;
}

void om_free(om_mesh *M) {
  free(M->coords); free(M->tets); free(M->nt_ptr); free(M->nt_idx); free(M->dL); free(M->adet); free(M->nbr);
  free(M->row_ptr); free(M->col_idx); free(M->K);
  for (int d = 0; d < 3; ++d) { free(M->G[d]); free(M->D[d]); }
  free(M->vol); free(M->b_of_node); free(M->node_of_b); free(M->tri); free(M->tri_normal);
  free(M->solid_angle); free(M->bem);
  memset(M, 0, sizeof(*M));
}

/* ---------------------------------------------------------------- operator export */

int om_export_operator(const om_mesh *M, int which, double coeff, int *rows, int *cols, int *nnz_out,
                       int32_t *rp, int32_t *ci, double *vals) {
  int N = M->n_nodes, nb = M->nb;
  const int32_t *R = M->row_ptr, *C = M->col_idx;
  int nr = 0, nc = 0; long long cnt = 0;
  switch (which) {
  case 0: /* (coeff) <d/dxj H_exch(k)||d/dxj m(k)>: row 3i+c, cols 3j+c */
    nr = 3 * N; nc = 3 * N;
    for (int i = 0; i < N; ++i) for (int c = 0; c < 3; ++c) {
      if (rp) rp[3 * i + c] = (int32_t)cnt;
      for (int k = R[i]; k < R[i + 1]; ++k) { if (ci) { ci[cnt] = 3 * C[k] + c; vals[cnt] = coeff * M->K[k]; } ++cnt; }
    }
    break;
  case 1: /* (coeff)<rho||d/dxj m(j)> + (coeff)<rho||D/Dxj m(j)>: row i, cols 3k+d */
    nr = N; nc = 3 * N;
    for (int i = 0; i < N; ++i) {
      if (rp) rp[i] = (int32_t)cnt;
      for (int k = R[i]; k < R[i + 1]; ++k) for (int d = 0; d < 3; ++d) { if (ci) { ci[cnt] = 3 * C[k] + d; vals[cnt] = coeff * M->D[d][k]; } ++cnt; }
    }
    break;
  case 2: /* <d/dxj rho || d/dxj phi> */
    nr = N; nc = N;
    for (int i = 0; i < N; ++i) {
      if (rp) rp[i] = (int32_t)cnt;
      for (int k = R[i]; k < R[i + 1]; ++k) { if (ci) { ci[cnt] = C[k]; vals[cnt] = coeff * M->K[k]; } ++cnt; }
    }
    break;
  case 3: /* -<H_demag(j) || d/dxj phi>: row 3i+d, cols k */
    nr = 3 * N; nc = N;
    for (int i = 0; i < N; ++i) for (int d = 0; d < 3; ++d) {
      if (rp) rp[3 * i + d] = (int32_t)cnt;
      for (int k = R[i]; k < R[i + 1]; ++k) { if (ci) { ci[cnt] = C[k]; vals[cnt] = -coeff * M->G[d][k]; } ++cnt; }
    }
    break;
  case 4: /* -<d/dxj phi[not outer] || d/dxj phi[not outer]>;phi[outer]=phi[outer] */
    nr = N; nc = N;
    for (int i = 0; i < N; ++i) {
      if (rp) rp[i] = (int32_t)cnt;
      if (M->b_of_node[i] >= 0) { if (ci) { ci[cnt] = i; vals[cnt] = 1.0; } ++cnt; continue; }
      for (int k = R[i]; k < R[i + 1]; ++k) {
        if (M->b_of_node[C[k]] >= 0) continue;
        if (ci) { ci[cnt] = C[k]; vals[cnt] = -coeff * M->K[k]; } ++cnt;
      }
    }
    break;
  case 5: /* <d/dxj phi[not outer] || d/dxj phi[outer]>;(L||R)=(*||phi[outer]) */
    nr = N; nc = nb;
    for (int i = 0; i < N; ++i) {
      if (rp) rp[i] = (int32_t)cnt;
      if (M->b_of_node[i] >= 0) continue;
      for (int k = R[i]; k < R[i + 1]; ++k) {
        int b = M->b_of_node[C[k]];
        if (b < 0) continue;
        if (ci) { ci[cnt] = b; vals[cnt] = coeff * M->K[k]; } ++cnt;
      }
    }
    break;
  default: return -1;
  }
  if (rp) rp[nr] = (int32_t)cnt;
  *rows = nr; *cols = nc; *nnz_out = (int)cnt;
  return 0;
}

/* ---------------------------------------------------------------- RHS */

int om_state_init(om_state *S, const om_mesh *M, const om_material *mat, const om_solver *nbc,
                  const om_solver *dbc, int do_demag, int nthreads) {
  memset(S, 0, sizeof(*S));
  S->M = M; S->mat = *mat; S->nbc = *nbc; S->dbc = *dbc; S->do_demag = do_demag; S->nthreads = nthreads;
  int N = M->n_nodes;
  S->phi1 = xcalloc(N, sizeof(double)); S->phi2 = xcalloc(N, sizeof(double)); S->phi = xcalloc(N, sizeof(double));
  S->rho = xcalloc(N, sizeof(double));
  S->h_ext = xcalloc(3 * (size_t)N, sizeof(double)); S->h_exch = xcalloc(3 * (size_t)N, sizeof(double));
  S->h_demag = xcalloc(3 * (size_t)N, sizeof(double)); S->h_anis = xcalloc(3 * (size_t)N, sizeof(double));
  S->h_total = xcalloc(3 * (size_t)N, sizeof(double)); S->dmdt = xcalloc(3 * (size_t)N, sizeof(double));
  S->tmp_b1 = xcalloc(M->nb, sizeof(double)); S->tmp_b2 = xcalloc(M->nb, sizeof(double));
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  return 0;
}

void om_state_free(om_state *S) {
  free(S->phi1); free(S->phi2); free(S->phi); free(S->rho); free(S->h_ext); free(S->h_exch); free(S->h_demag);
  free(S->h_anis); free(S->h_total); free(S->dmdt); free(S->tmp_b1); free(S->tmp_b2);
  for (int k = 0; k < 2; ++k) { free(S->basis_b[k]); free(S->basis_x[k]); }
  free(S->an_epow); free(S->an_hpow); free(S->an_ecoef); free(S->an_hcoef);
  free(S->stt_j); free(S->stt_dmdc); free(S->pin);
  memset(S, 0, sizeof(*S));
}

int om_set_pinning(om_state *S, const double *pin) {
  const int N = S->M->n_nodes;
  free(S->pin);
  S->pin = NULL;
  if (pin) { S->pin = xcalloc(N, sizeof(double)); memcpy(S->pin, pin, sizeof(double) * N); }
  return 0;
}

int om_set_stt(om_state *S, double c4, double c5, const double *j) {
  const int N = S->M->n_nodes;
  if (!S->stt_j) { S->stt_j = xcalloc(3 * (size_t)N, sizeof(double)); S->stt_dmdc = xcalloc(3 * (size_t)N, sizeof(double)); }
  if (j) memcpy(S->stt_j, j, sizeof(double) * 3 * N);
  else memset(S->stt_j, 0, sizeof(double) * 3 * N);
  S->stt_c4 = c4; S->stt_c5 = c5;
  return 0;
}

/* set_dm_dcurrent (nmag_lam.py:892-903): SM*V op_grad_m, site-wise
 * grad_m(i,j) current_density(j), CFBOX. */
static void dm_dcurrent(const om_state *S, const double *m, double *out) {
  const om_mesh *M = S->M;
  const int N = M->n_nodes;
  for (int a = 0; a < N; ++a) {
    double g[3][3] = {{0}};
    for (int k = M->row_ptr[a]; k < M->row_ptr[a + 1]; ++k) {
      const double *mb = m + 3 * (size_t)M->col_idx[k];
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) g[c][d] += M->G[d][k] * mb[c];
    }
    const double *J = S->stt_j + 3 * (size_t)a;
    for (int c = 0; c < 3; ++c) out[3 * (size_t)a + c] = ((g[c][0] * J[0] + g[c][1] * J[1]) + g[c][2] * J[2]) / M->vol[a];
  }
}

int om_set_anisotropy_poly(om_state *S, int ne, const int32_t *epow, const double *ecoef, int nh,
                           const int32_t *hpow, const double *hcoef) {
  if (ne < 0 || nh < 0) return -1;
  free(S->an_epow); free(S->an_hpow); free(S->an_ecoef); free(S->an_hcoef);
  S->an_epow = xcalloc(ne + 1, sizeof(int32_t)); S->an_ecoef = xcalloc(ne + 1, sizeof(double));
  S->an_hpow = xcalloc(nh + 1, sizeof(int32_t)); S->an_hcoef = xcalloc(3 * (size_t)nh + 1, sizeof(double));
  if (ne) { memcpy(S->an_epow, epow, sizeof(int32_t) * ne); memcpy(S->an_ecoef, ecoef, sizeof(double) * ne); }
  if (nh) { memcpy(S->an_hpow, hpow, sizeof(int32_t) * nh); memcpy(S->an_hcoef, hcoef, sizeof(double) * 3 * nh); }
  S->an_ne = ne; S->an_nh = nh;
  return 0;
}

/* One generated polynomial: sum over the terms with a non-zero coefficient
 * (stride apart in coef) of (c)*m(0)^a*m(1)^b*m(2)^c, multiplied left to
 * right, summed in order. */
static double poly_eval(int nt, const int32_t *pw, const double *coef, int stride, const double *m) {
  double sum = 0.0;
  for (int t = 0; t < nt; ++t) {
    const double c = coef[(size_t)t * stride];
    if (c == 0.0) continue;
    double v = c;
    const int e[3] = {pw[t] & 15, (pw[t] >> 4) & 15, (pw[t] >> 8) & 15};
    for (int d = 0; d < 3; ++d)
      for (int k = 0; k < e[d]; ++k) v *= m[d];
    sum += v;
  }
  return sum;
}

/* Sparse A x where A is K restricted by a mask: mode 0 = full K; mode 1 =
 * Dirichlet operator K_II (+) I_B (the sign-flipped op_laplace_DBC). */
static void spmv_K(const om_mesh *M, int mode, const double *x, double *y) {
  int N = M->n_nodes;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < N; ++i) {
    if (mode == 1 && M->b_of_node[i] >= 0) { y[i] = x[i]; continue; }
    double s = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      int j = M->col_idx[k];
      if (mode == 1 && M->b_of_node[j] >= 0) continue;
      s += M->K[k] * x[j];
    }
    y[i] = s;
  }
}

static double dot(int n, const double *a, const double *b) {
  double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) schedule(static)
#endif
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Least squares (G + 1e-12 diag G) c = v by Cholesky; nearly dependent
 * directions (collapsed pivots) get c = 0.  Same algorithm as the device. */
static void small_solve(int n, const double *G, const double *v, double *c) {
  double L[OM_BASIS][OM_BASIS], y[OM_BASIS];
  int on[OM_BASIS];
  for (int i = 0; i < n; ++i) {
    on[i] = 1;
    for (int j = 0; j <= i; ++j) {
      double s = G[i * OM_BASIS + j];
      if (i == j) s *= 1.0 + 1e-12;
      for (int k = 0; k < j; ++k) if (on[k]) s -= L[i][k] * L[j][k];
      if (i == j) {
        if (!(s > 1e-14 * G[i * OM_BASIS + i]) || !on[i]) { on[i] = 0; L[i][i] = 1.0; }
        else L[i][i] = sqrt(s);
      } else {
        L[i][j] = on[j] ? s / L[j][j] : 0.0;
      }
    }
    if (!on[i]) for (int j = 0; j < i; ++j) L[i][j] = 0.0;
  }
  for (int i = 0; i < n; ++i) {
    double s = v[i];
    for (int k = 0; k < i; ++k) s -= L[i][k] * y[k];
    y[i] = on[i] ? s / L[i][i] : 0.0;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < n; ++k) s -= L[k][i] * c[k];
    c[i] = on[i] ? s / L[i][i] : 0.0;
  }
}

/* Jacobi-preconditioned CG, stop when ||r||_2 <= max(rtol ||b||_2, atol)
 * (PETSc's default test measured on ||b||).  mode 0 projects the constant
 * null space of the Neumann operator out of b and of the solution
 * (nullspace_subfields=["phi"], nmag_lam.py:623-624).
 * Initial guess: the reference warm-starts from the previous solution
 * (initial_guess_nonzero, nmag_lam.py:617,628); here b is first projected
 * onto the span of the last OM_BASIS right-hand sides of this solve kind and
 * x starts from the same combination of their solutions (the previous
 * solution when the basis is empty).  Returns iterations, or -1. */
static int pcg(om_state *S, int mode, const double *b_in, double *x, double rtol, double atol, int maxits) {
  const om_mesh *M = S->M;
  int N = M->n_nodes;
  double *r = malloc(sizeof(double) * N), *z = malloc(sizeof(double) * N), *p = malloc(sizeof(double) * N),
         *q = malloc(sizeof(double) * N), *dinv = malloc(sizeof(double) * N), *b = malloc(sizeof(double) * N);
  memcpy(b, b_in, sizeof(double) * N);
  for (int i = 0; i < N; ++i) {
    double dg = 1.0;
    if (!(mode == 1 && M->b_of_node[i] >= 0)) {
      int pos = row_find(M->col_idx, M->row_ptr[i], M->row_ptr[i + 1], i);
      dg = M->K[pos];
    }
    dinv[i] = 1.0 / dg;
  }
  if (mode == 0) {
    double mb = 0.0; for (int i = 0; i < N; ++i) mb += b[i]; mb /= N;
    for (int i = 0; i < N; ++i) b[i] -= mb;
  }
  if (!S->basis_b[mode]) {
    S->basis_b[mode] = xcalloc((size_t)OM_BASIS * N, sizeof(double));
    S->basis_x[mode] = xcalloc((size_t)OM_BASIS * N, sizeof(double));
  }
  const int count = S->bcount[mode], head = S->bhead[mode];
  double bdot[OM_BASIS];
  for (int j = 0; j < count; ++j) bdot[j] = dot(N, b, S->basis_b[mode] + (size_t)j * N);
  double bb = dot(N, b, b);
  if (count > 0) {
    double c[OM_BASIS];
    small_solve(count, S->gram[mode], bdot, c);
    for (int i = 0; i < N; ++i) {
      double g = 0.0;
      for (int j = 0; j < count; ++j) g += c[j] * S->basis_x[mode][(size_t)j * N + i];
      x[i] = (mode == 1 && M->b_of_node[i] >= 0) ? b[i] : g;
    }
  }
  double bnorm = sqrt(bb);
  double tol = rtol * bnorm; if (atol > tol) tol = atol;
  spmv_K(M, mode, x, q);
  for (int i = 0; i < N; ++i) r[i] = b[i] - q[i];
  double rnorm = sqrt(dot(N, r, r));
  int it = 0, status = 0;
  double rz = 0.0;
  while (rnorm > tol) {
    if (it >= maxits) { status = -1; break; }
    for (int i = 0; i < N; ++i) z[i] = dinv[i] * r[i];
    double rz_new = dot(N, r, z);
    if (it == 0) { memcpy(p, z, sizeof(double) * N); }
    else { double beta = rz_new / rz; for (int i = 0; i < N; ++i) p[i] = z[i] + beta * p[i]; }
    rz = rz_new;
    spmv_K(M, mode, p, q);
    double alpha = rz / dot(N, p, q);
    for (int i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    rnorm = sqrt(dot(N, r, r));
    ++it;
  }
  if (mode == 0) { double mx = 0.0; for (int i = 0; i < N; ++i) mx += x[i]; mx /= N; for (int i = 0; i < N; ++i) x[i] -= mx; }
  /* remember (b, x) in the ring and update the Gram matrix */
  memcpy(S->basis_b[mode] + (size_t)head * N, b, sizeof(double) * N);
  memcpy(S->basis_x[mode] + (size_t)head * N, x, sizeof(double) * N);
  int ncount = count < OM_BASIS ? count + 1 : OM_BASIS;
  for (int j = 0; j < ncount; ++j) {
    double g = (j == head) ? bb : bdot[j];
    S->gram[mode][head * OM_BASIS + j] = g;
    S->gram[mode][j * OM_BASIS + head] = g;
  }
  S->bcount[mode] = ncount;
  S->bhead[mode] = (head + 1) % OM_BASIS;
  free(r); free(z); free(p); free(q); free(dinv); free(b);
  return status < 0 ? -1 : it;
}

/* set_H_demag (nmag_lam.py:740-760) */
static int demag(om_state *S, const double *m) {
  const om_mesh *M = S->M;
  int N = M->n_nodes, nb = M->nb;
  double Ms = S->mat.Ms;
  /* rho = -(op_div_m m)  */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < N; ++i) {
    double s = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      const double *mj = m + 3 * (size_t)M->col_idx[k];
      s += (M->D[0][k] * mj[0] + M->D[1][k] * mj[1]) + M->D[2][k] * mj[2];
    }
    S->rho[i] = -(Ms * s);
  }
  int it1 = pcg(S, 0, S->rho, S->phi1, S->nbc.rtol, S->nbc.atol, S->nbc.maxits);
  S->last_iters_nbc = it1;
  if (it1 < 0) return 1;
  /* phi2b = BEM phi1b */
  for (int b = 0; b < nb; ++b) S->tmp_b1[b] = S->phi1[M->node_of_b[b]];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int k = 0; k < nb; ++k) {
    const double *row = M->bem + (size_t)k * nb;
    double s = 0.0;
    for (int c = 0; c < nb; ++c) s += row[c] * S->tmp_b1[c];
    S->tmp_b2[k] = s;
  }
  /* Dirichlet solve: K_II phi2_I = -K_IB phi2b, boundary rows = phi2b */
  double *rhs = malloc(sizeof(double) * N);
  for (int i = 0; i < N; ++i) {
    int bi = M->b_of_node[i];
    if (bi >= 0) { rhs[i] = S->tmp_b2[bi]; S->phi2[i] = S->tmp_b2[bi]; continue; }
    double s = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      int b = M->b_of_node[M->col_idx[k]];
      if (b >= 0) s += M->K[k] * S->tmp_b2[b];
    }
    rhs[i] = -s;
  }
  int it2 = pcg(S, 1, rhs, S->phi2, S->dbc.rtol, S->dbc.atol, S->dbc.maxits);
  free(rhs);
  S->last_iters_dbc = it2;
  if (it2 < 0) return 2;
  for (int i = 0; i < N; ++i) S->phi[i] = S->phi1[i] + S->phi2[i];
  /* H_demag = (op_grad_phi phi) / V */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < N; ++i) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      double p = S->phi[M->col_idx[k]];
      s0 += M->G[0][k] * p; s1 += M->G[1][k] * p; s2 += M->G[2][k] * p;
    }
    double V = M->vol[i];
    S->h_demag[3 * i] = -s0 / V; S->h_demag[3 * i + 1] = -s1 / V; S->h_demag[3 * i + 2] = -s2 / V;
  }
  return 0;
}

static void exch(const om_state *S, const double *m, double *h) {
  const om_mesh *M = S->M;
  int N = M->n_nodes;
  double c = S->mat.exch_coeff;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < N; ++i) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      const double *mj = m + 3 * (size_t)M->col_idx[k];
      double kv = M->K[k];
      s0 += kv * mj[0]; s1 += kv * mj[1]; s2 += kv * mj[2];
    }
    double V = M->vol[i];
    h[3 * i] = -c * s0 / V; h[3 * i + 1] = -c * s1 / V; h[3 * i + 2] = -c * s2 / V;
  }
}

/* LLG local equation (nmag_lam.py:417-430):
   dm/dt = C1 m x H + C2 m x (m x H) + C3 (1 - m.m) m   (pin = 1). */
static inline void llg(const double *m, const double *H, double C1, double C2, double C3, double *out) {
  double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
  double mxmxH[3] = {m[1] * mxH[2] - m[2] * mxH[1], m[2] * mxH[0] - m[0] * mxH[2], m[0] * mxH[1] - m[1] * mxH[0]};
  double c3 = C3 * (1.0 - ((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]));
  for (int d = 0; d < 3; ++d) out[d] = (C1 * mxH[d] + C2 * mxmxH[d]) + c3 * m[d];
}

int om_rhs(om_state *S, const double *m, double *dmdt_out) {
  const om_mesh *M = S->M;
  int N = M->n_nodes;
  int st = 0;
  if (S->do_demag) st = demag(S, m);
  else memset(S->h_demag, 0, sizeof(double) * 3 * N);
  if (st) return st;
  exch(S, m, S->h_exch);
  const om_material *mt = &S->mat;
  const int stt = S->stt_j && (S->stt_c4 != 0.0 || S->stt_c5 != 0.0);
  if (stt) dm_dcurrent(S, m, S->stt_dmdc);
  for (int i = 0; i < N; ++i) {
    const double *mi = m + 3 * (size_t)i;
    double *ha = S->h_anis + 3 * (size_t)i;
    if (mt->K1 != 0.0) {
      double am = (mt->axis[0] * mi[0] + mt->axis[1] * mi[1]) + mt->axis[2] * mi[2];
      for (int d = 0; d < 3; ++d) ha[d] = mt->anis_coeff * am * (mt->axis[d] - am * mi[d]);
    } else ha[0] = ha[1] = ha[2] = 0.0;
    if (S->an_nh)
      for (int d = 0; d < 3; ++d) ha[d] += poly_eval(S->an_nh, S->an_hpow, S->an_hcoef + d, 3, mi);
    double *ht = S->h_total + 3 * (size_t)i;
    for (int d = 0; d < 3; ++d)
      ht[d] = ((S->h_ext[3 * i + d] + S->h_exch[3 * i + d]) + ha[d]) + S->h_demag[3 * i + d];
    llg(mi, ht, mt->C1, mt->C2, mt->C3, S->dmdt + 3 * (size_t)i);
    if (stt) {   /* + C4 m x (m x u) + C5 m x u, after the C1..C3 terms */
      const double *u = S->stt_dmdc + 3 * (size_t)i;
      double mxu[3] = {mi[1] * u[2] - mi[2] * u[1], mi[2] * u[0] - mi[0] * u[2], mi[0] * u[1] - mi[1] * u[0]};
      double mxmxu[3] = {mi[1] * mxu[2] - mi[2] * mxu[1], mi[2] * mxu[0] - mi[0] * mxu[2],
                         mi[0] * mxu[1] - mi[1] * mxu[0]};
      double *o = S->dmdt + 3 * (size_t)i;
      for (int d = 0; d < 3; ++d) o[d] = (o[d] + S->stt_c4 * mxmxu[d]) + S->stt_c5 * mxu[d];
    }
    if (S->pin) for (int d = 0; d < 3; ++d) S->dmdt[3 * (size_t)i + d] *= S->pin[i];
  }
  if (dmdt_out) memcpy(dmdt_out, S->dmdt, sizeof(double) * 3 * N);
  S->n_rhs++;
  return 0;
}

/* local_E_total (nmag_lam.py:454-460): densities per node. */
int om_energy_density(const om_state *S, const double *m, double *E5) {
  int N = S->M->n_nodes;
  const om_material *mt = &S->mat;
  for (int i = 0; i < N; ++i) {
    const double *mi = m + 3 * (size_t)i;
    const double *hx = S->h_exch + 3 * i, *hd = S->h_demag + 3 * i, *he = S->h_ext + 3 * i;
    double e_ex = mt->E_coeff_half * ((mi[0] * hx[0] + mi[1] * hx[1]) + mi[2] * hx[2]);
    double e_dm = mt->E_coeff_half * ((mi[0] * hd[0] + mi[1] * hd[1]) + mi[2] * hd[2]);
    double e_ext = mt->E_coeff_ext * ((mi[0] * he[0] + mi[1] * he[1]) + mi[2] * he[2]);
    double e_an = 0.0;
    if (mt->K1 != 0.0) {
      double am = (mt->axis[0] * mi[0] + mt->axis[1] * mi[1]) + mt->axis[2] * mi[2];
      e_an = -mt->K1 * am * am;
    }
    if (S->an_ne) e_an += poly_eval(S->an_ne, S->an_epow, S->an_ecoef, 1, mi);
    E5[i] = e_ex; E5[N + i] = e_dm; E5[2 * N + i] = e_ext; E5[3 * N + i] = e_an;
    E5[4 * N + i] = ((e_dm + e_ex) + e_ext) + e_an;
  }
  return 0;
}

/* Jacobian of C1 m x H + C2 m x (m x H) with H frozen (PRIMARY) plus
 * dH/dm = op_H_exch / V (OPERATOR) -- nmag_lam.py:432-436,684-704,
 * nsim.ml:967-1050.  No C3 term, no demag, no anisotropy, as the reference. */
void om_jv(const om_state *S, const double *mJ, const double *HJ, const double *v, double *out) {
  const om_mesh *M = S->M;
  int N = M->n_nodes;
  double c = S->mat.exch_coeff, C1 = S->mat.C1, C2 = S->mat.C2;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < N; ++i) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k) {
      const double *vj = v + 3 * (size_t)M->col_idx[k];
      double kv = M->K[k];
      s0 += kv * vj[0]; s1 += kv * vj[1]; s2 += kv * vj[2];
    }
    double V = M->vol[i];
    double hv[3] = {-c * s0 / V, -c * s1 / V, -c * s2 / V};
    const double *m = mJ + 3 * (size_t)i, *H = HJ + 3 * (size_t)i, *w = v + 3 * (size_t)i;
    /* d/dm [m x H] . w = w x H ; d/dH [m x H] . hv = m x hv */
    double a[3] = {w[1] * H[2] - w[2] * H[1] + (m[1] * hv[2] - m[2] * hv[1]),
                   w[2] * H[0] - w[0] * H[2] + (m[2] * hv[0] - m[0] * hv[2]),
                   w[0] * H[1] - w[1] * H[0] + (m[0] * hv[1] - m[1] * hv[0])};
    /* d[m x (m x H)] = w x (m x H) + m x (w x H) + m x (m x hv) */
    double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
    double wxH[3] = {w[1] * H[2] - w[2] * H[1], w[2] * H[0] - w[0] * H[2], w[0] * H[1] - w[1] * H[0]};
    double mxhv[3] = {m[1] * hv[2] - m[2] * hv[1], m[2] * hv[0] - m[0] * hv[2], m[0] * hv[1] - m[1] * hv[0]};
    double t1[3] = {w[1] * mxH[2] - w[2] * mxH[1], w[2] * mxH[0] - w[0] * mxH[2], w[0] * mxH[1] - w[1] * mxH[0]};
    double u[3] = {wxH[0] + mxhv[0], wxH[1] + mxhv[1], wxH[2] + mxhv[2]};
    double t2[3] = {m[1] * u[2] - m[2] * u[1], m[2] * u[0] - m[0] * u[2], m[0] * u[1] - m[1] * u[0]};
    for (int d = 0; d < 3; ++d) out[3 * i + d] = C1 * a[d] + C2 * (t1[d] + t2[d]);
    if (S->pin) for (int d = 0; d < 3; ++d) out[3 * i + d] *= S->pin[i];
  }
}

/* One Lindholm evaluation for an explicit triangle (test hook): the same
 * arithmetic as the fill, with geo_eps = 1e-13 * max |coordinate|. */
void om_lindholm_single(const double *p0, const double *p1, const double *p2, const double *normal,
                        const double *obs, double *lh) {
  om_mesh M;
  memset(&M, 0, sizeof(M));
  double coords[9]; int32_t node_of_b[3] = {0, 1, 2}; int32_t tri[3] = {0, 1, 2};
  double nrm[3] = {normal[0], normal[1], normal[2]};
  memcpy(coords, p0, 3 * sizeof(double)); memcpy(coords + 3, p1, 3 * sizeof(double)); memcpy(coords + 6, p2, 3 * sizeof(double));
  M.coords = coords; M.node_of_b = node_of_b; M.tri = tri; M.tri_normal = nrm; M.ntri = 1;
  om_tri_geo g;
  tri_setup(&M, 0, &g);
  double mg = g.maxgeo;
  for (int d = 0; d < 3; ++d) if (fabs(obs[d]) > mg) mg = fabs(obs[d]);
  lh[0] = lh[1] = lh[2] = 0.0;
  if (g.ok) lindholm(&g, obs, mg * 1e-13, lh);
}
