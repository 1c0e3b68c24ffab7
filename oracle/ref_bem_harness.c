/* ref_bem_harness.c -- drives the reference's own Lindholm stub,
 * caml_bem3d_raw_lindholm_block_pbc (src/bem3d_stubs.c:413-610, compiled
 * unmodified against oracle/caml_shim), to fill a dense BEM matrix the way
 * the reference's row fill does (src/bem3d.ml:938-1047).
 *
 * TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by oracle/Makefile when
 * the reference tree is present, and used by tests/ to pin the oracle's and
 * the device's BEM matrices to the reference's own arithmetic.
 *
 * The fill, as bem3d.ml:938-1047 runs it for a mesh without periodic copies:
 * for each surface triangle in the given order, one stub call evaluates the
 * triangle against every observer (one row per boundary node, rows in
 * short-vector order), with the identity transformation, one grey factor of
 * 1.0 and one zero displacement (bem3d.ml:979, the lattice_info = None case),
 * min_dist = 0.0 (its default); the three weights of each row are then added
 * to the row's entries at the triangle's three vertex columns
 * (fun_add_contrib).  After all triangles, each diagonal entry gets
 * solid_angle / (4 pi) - 1 (bem3d.ml:1040-1043). */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "caml/mlvalues.h"

value caml_bem3d_raw_lindholm_block_pbc(value ml_min_dist, value ml_args);

/* A block of n words with its header, as the stub expects (see mlvalues.h). */
static value *new_block(size_t n) {
  value *b = (value *)calloc(n + 1, sizeof(value));
  if (!b) return NULL;
  b[0] = (value)n;
  return b + 1;
}
static void free_block(value *v) {
  if (v) free(v - 1);
}
static value *new_floats(size_t n, const double *src) {
  value *b = new_block(n);
  if (b && src) memcpy(b, src, n * sizeof(double));
  return b;
}

/* bem (nb x nb, row-major, overwritten): the reference's BEM matrix for
 * observers obs (nb x 3, the boundary nodes in short-vector order), surface
 * triangles tri (ntri x 3 boundary indices, in the fill's visiting order)
 * with outward normals nrm (ntri x 3), and interior solid angles (nb).
 * Returns 0, or -1 if memory runs out. */
int ref_fill_bem(int nb, const double *obs, int ntri, const int32_t *tri, const double *nrm,
                 const double *solid_angle, double *bem) {
  const double pi = 3.141592653589793238462643383279502884;
  const double zero3[3] = {0.0, 0.0, 0.0};
  const double identity[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  const double one = 1.0, min_dist = 0.0;
  int rc = -1;
  size_t k;
  value *observers = new_block((size_t)nb), *otrans = new_block(3), *grey = new_floats(1, &one);
  value *disp = new_block(1), *store = new_block(3), *args = new_block(9);
  value *p[3] = {NULL, NULL, NULL}, *osn = new_floats(3, NULL);
  if (!observers || !otrans || !grey || !disp || !store || !args || !osn) goto out;
  memset(observers, 0, sizeof(value) * (size_t)nb);
  for (k = 0; k < (size_t)nb; ++k)
    if (!(observers[k] = (value)new_floats(3, obs + 3 * k))) goto out;
  for (k = 0; k < 3; ++k) {
    if (!(otrans[k] = (value)new_floats(3, identity[k]))) goto out;
    if (!(store[k] = (value)new_floats((size_t)nb, NULL))) goto out;
    if (!(p[k] = new_floats(3, NULL))) goto out;
  }
  if (!(disp[0] = (value)new_floats(3, zero3))) goto out;
  args[0] = (value)p[0];
  args[1] = (value)p[1];
  args[2] = (value)p[2];
  args[3] = (value)osn;
  args[4] = (value)store;
  args[5] = (value)otrans;
  args[6] = (value)grey;
  args[7] = (value)disp;
  args[8] = (value)observers;
  memset(bem, 0, sizeof(double) * (size_t)nb * (size_t)nb);
  for (int t = 0; t < ntri; ++t) {
    const int32_t *tv = tri + 3 * (size_t)t;
    for (int c = 0; c < 3; ++c) memset((double *)store[c], 0, sizeof(double) * (size_t)nb);
    for (int c = 0; c < 3; ++c) memcpy(p[c], obs + 3 * (size_t)tv[c], 3 * sizeof(double));
    memcpy(osn, nrm + 3 * (size_t)t, 3 * sizeof(double));
    caml_bem3d_raw_lindholm_block_pbc((value)&min_dist, (value)args);
    for (int c = 0; c < 3; ++c) {
      const double *lh = (const double *)store[c];
      for (k = 0; k < (size_t)nb; ++k) bem[k * (size_t)nb + (size_t)tv[c]] += lh[k];
    }
  }
  for (k = 0; k < (size_t)nb; ++k) bem[k * (size_t)nb + k] += solid_angle[k] / (4.0 * pi) - 1.0;
  rc = 0;
out:
  if (observers)
    for (k = 0; k < (size_t)nb; ++k) free_block((value *)observers[k]);
  for (k = 0; k < 3; ++k) {
    if (otrans) free_block((value *)otrans[k]);
    if (store) free_block((value *)store[k]);
    free_block(p[k]);
  }
  if (disp) free_block((value *)disp[0]);
  free_block(observers); free_block(otrans); free_block(grey); free_block(disp);
  free_block(store); free_block(args); free_block(osn);
  return rc;
}
