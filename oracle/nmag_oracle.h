/*
 * nmag_oracle.h -- CPU restatement of nmag/nsim's LLG right-hand side and its
 * time integration, used ONLY as test infrastructure: the reference results of
 * the CUDA library's parity tests and the timed CPU baseline of bench.py.  Nothing in
 * the product links, imports or calls this code.
 *
 * Parity status: the reference as a whole (OCaml + Python 2 + PETSc 2.3.3 +
 * SUNDIALS CVODE 2.3.0) cannot be built or run here, and the reference tree
 * holds no golden vectors for this path.  Its one plain-C piece on the path,
 * the Lindholm stub src/bem3d_stubs.c, is compiled unmodified against a
 * minimal caml shim (ref_bem_harness.c, oracle/_ref): om_fill_bem equals its
 * fill bit for bit.  The rest is pinned against known-answer invariants
 * (uniform-m exchange field, cube demag factor 1/3, BEM row sums,
 * single-spin LLG solution, SI<->su conversions).
 *
 * Every routine cites the reference file:line it restates (paths relative to
 * the nmag-src project root).
 */
#ifndef NMAG_ORACLE_H
#define NMAG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_mesh {
  int n_nodes, n_tets;
  double *coords;        /* 3N, copied */
  int32_t *tets;         /* 4T, copied */
  /* node -> tet adjacency, tets ascending (fem.ml:2523-2577 keeps simplices of a site ascending) */
  int32_t *nt_ptr, *nt_idx;
  /* per-tet geometry: barycentric gradients dL[t][a][d] and |det| of the point matrix */
  double *dL, *adet;
  /* face neighbours: nbr[4t+f] is the tet across the face opposite local vertex f, -1 = outer face */
  int32_t *nbr;
  /* scalar P1 CSR pattern (N + 2*edges entries), columns ascending */
  int nnz;
  int32_t *row_ptr, *col_idx;
  double *K;             /* int grad phi_i . grad phi_j                   */
  double *G[3];          /* int phi_i d_d phi_j                           */
  double *D[3];          /* G_d minus the outer-surface term (div of m)   */
  double *vol;           /* box volumes V_i = int phi_i                   */
  /* boundary ("phi[outer]") short vector, ascending node order */
  int nb;
  int32_t *b_of_node, *node_of_b;
  /* surface triangles in the order the reference's fill loop visits them */
  int ntri;
  int32_t *tri;          /* 3*ntri short indices */
  double *tri_normal;    /* 3*ntri outward unit normals */
  double *solid_angle;   /* nb interior solid angles */
  double *bem;           /* nb*nb row-major, filled by om_fill_bem */
} om_mesh;

/* Build topology, CSR pattern, P1 values, boundary data (no BEM fill). 0 = ok. */
int om_build(om_mesh *M, int n_nodes, const double *coords, int n_tets, const int32_t *tets);
/* Lindholm BEM fill (bem3d.ml:938-1047 + bem3d_stubs.c:413-610). */
int om_fill_bem(om_mesh *M, int nthreads);
void om_free(om_mesh *M);

/* Reference-shaped CSR export of the six operators (nmag_lam.py:569-606).
 * which: 0 op_H_exch (3N x 3N), 1 op_div_m (N x 3N), 2 op_neg_laplace_phi (N x N),
 *        3 op_grad_phi (3N x N), 4 op_laplace_DBC (N x N), 5 op_load_DBC (N x Nb).
 * Call with NULL arrays to get sizes (rows, nnz); then with arrays. */
int om_export_operator(const om_mesh *M, int which, double coeff, int *rows, int *cols, int *nnz,
                       int32_t *row_ptr, int32_t *col_idx, double *vals);

/* Material in simulation units (main.py:347-465). */
typedef struct om_material {
  double Ms, exch_coeff;            /* su_Ms, su_exch_prefactor (2A/(mu0 Ms)) */
  double C1, C2, C3;                /* LLG coefficients as the local equation sees them */
  double K1, axis[3], anis_coeff;   /* uniaxial anisotropy; anis_coeff = 2 K1/(mu0 Ms) */
  double E_coeff_half, E_coeff_ext; /* -0.5 Ms mu0 and -1.0 Ms mu0 (energy densities) */
} om_material;

/* Solver tolerances for the two Poisson solves (nmag_lam.py:614-634). */
typedef struct om_solver {
  double rtol, atol; int maxits;
} om_solver;

#define OM_BASIS 10

typedef struct om_state {
  const om_mesh *M;
  om_material mat;
  om_solver nbc, dbc;
  int do_demag;
  double *phi1, *phi2;   /* warm-start state of the two solves, N each */
  double *h_ext;         /* 3N */
  /* scratch / outputs of the last evaluation */
  double *h_exch, *h_demag, *h_anis, *h_total, *rho, *phi, *dmdt;
  double *tmp_b1, *tmp_b2;
  int last_iters_nbc, last_iters_dbc;
  long long n_rhs;
  int nthreads;
  /* initial-guess basis of each solve kind: last OM_BASIS right-hand sides
     and solutions, their Gram matrix, {count, head} */
  double *basis_b[2], *basis_x[2];
  double gram[2][OM_BASIS * OM_BASIS];
  int bcount[2], bhead[2];
  /* anisotropy in polynomial form (om_set_anisotropy_poly); owned copies */
  int an_ne, an_nh;
  int32_t *an_epow, *an_hpow;
  double *an_ecoef, *an_hcoef;
  /* spin-transfer torque (om_set_stt): LLG_C4, LLG_C5, current density (3N,
     owned) and the last dm_dcurrent (3N) */
  double stt_c4, stt_c5;
  double *stt_j, *stt_dmdc;
  double *pin;   /* N, owned; NULL = 1 everywhere (om_set_pinning) */
} om_state;


int om_state_init(om_state *S, const om_mesh *M, const om_material *mat, const om_solver *nbc,
                  const om_solver *dbc, int do_demag, int nthreads);
void om_state_free(om_state *S);
/* Anisotropy as the polynomials the reference generates for it
 * (nsim_anisotropy.ml:189-236, equations E_anis and H_anis(d) of
 * nmag_lam.py:485-502): E = sum_t e_t m^p_t, H_d = sum_t h_{t,d} m^p_t with
 * exponents packed a | b << 4 | c << 8; added to the closed-form K1 term.
 * Evaluated like the generated C: per component, terms in table order,
 * each (c)*m(0)*...*m(2) left to right.  ne = nh = 0 removes it. */
int om_set_anisotropy_poly(om_state *S, int ne, const int32_t *epow, const double *ecoef, int nh,
                           const int32_t *hpow, const double *hcoef);
/* Spin-transfer torque (nmag_lam.py:417-424,872-903): dm/dt gains
 * c4 m x (m x u) + c5 m x u, u = dm_dcurrent computed each RHS as
 * op_grad_m (G_d m_c, no sign), site-wise grad_m(c,d) J(d) summed over d in
 * order, then divided by the box volume.  j: 3N current density (NULL =
 * zero). */
int om_set_stt(om_state *S, double c4, double c5, const double *j);
/* Pinning field (nmag_lam.py:417-436): every dm/dt term and the Jacobian
 * rows carry the factor pin of their node.  NULL = 1 everywhere. */
int om_set_pinning(om_state *S, const double *pin);
/* Full RHS: H_exch, H_demag (FEM/BEM), H_anis, H_total, dm/dt (nmag_lam.py:734-832). */
int om_rhs(om_state *S, const double *m, double *dmdt_out);
/* Energy densities E_exch, E_demag, E_ext, E_anis, E_total (5 x N) from the last fields. */
int om_energy_density(const om_state *S, const double *m, double *E5);
/* Matrix-free Jacobian-vector product with frozen (mJ, HJ) (nsim.ml:967-1050, 2315-2417). */
void om_jv(const om_state *S, const double *mJ, const double *HJ, const double *v, double *out);

/* CVODE-style BDF (orders 1..qmax), Newton + left-preconditioned GMRES. */
typedef struct om_ts_stats {
  long long nst, nfe, nni, nli, ncfn, netf, npe, nps, njv, nje;
  double hcur, tcur; int qcur;
} om_ts_stats;

typedef struct om_bdf om_bdf;
om_bdf *om_bdf_create(om_state *S, int qmax, int maxl, double rtol, double atol,
                      double pc_rtol, double pc_atol);
void om_bdf_free(om_bdf *B);
int om_bdf_init(om_bdf *B, double t0, const double *m0);
/* Advance to tout (CV_NORMAL, interpolated output) or stop exactly at tout (tstop). */
int om_bdf_advance(om_bdf *B, double tout, int exact_tstop, long long max_steps, double *t_reached,
                   double *m_out);
void om_bdf_stats(const om_bdf *B, om_ts_stats *st);
/* Preconditioner of the Newton systems: kind 0 (default) one exact 3x3
 * block-Jacobi sweep; kind 1 the reference's (nsim.ml:2210-2262,2419-2483):
 * P = I - gamma J assembled, GMRES(restart) with ILU(0), to pc_rtol/pc_atol
 * or maxit iterations (restart, maxit < 1: PETSc's 30, 10000). */
void om_bdf_set_precond(om_bdf *B, int kind, int restart, int maxit);
long long om_bdf_pc_iterations(const om_bdf *B);
/* Test hook: out = (I - gamma J(mJ, HJ)) v from the assembled matrix. */
void om_pc_matrix_apply(const om_state *S, const double *mJ, const double *HJ, double gamma, const double *v,
                        double *out);

/* Fixed-step RK4 (differentiation form forward). */
int om_rk4(om_state *S, double *m, double dt, int nsteps);

/* Shape-quality helpers used by tests. */
double om_triangle_space_angle(const double *obs, const double *p0, const double *p1, const double *p2);
void om_lindholm_single(const double *p0, const double *p1, const double *p2, const double *normal,
                        const double *obs, double *lh);

#ifdef __cplusplus
}
#endif
#endif
