/*
 * nmag_bdf.c -- CPU restatement (test infrastructure only) of the time
 * integrator behind nsim's timestepper: SUNDIALS CVODE 2.3.0 as configured in
 * nsim.ml:2485-2535 and sundials_sp_stubs.c:780-1030 -- BDF (CV_BDF), Newton
 * iteration (CV_NEWTON), SPGMR with left preconditioning (maxl = krylov_max),
 * scalar rtol/atol, max order 2 by default, CV_NORMAL_TSTOP when exact_tstop.
 *
 * SUNDIALS is not vendored in the reference tree (dlopen'd at
 * sundials_sp_stubs.c:115-150); this file restates the published method
 * (Hindmarsh et al., "SUNDIALS: Suite of nonlinear and differential/algebraic
 * equation solvers", ACM TOMS 31 (2005); Cohen & Hindmarsh, "CVODE, a
 * stiff/nonstiff ODE solver in C", Computers in Physics 10 (1996)): the
 * fixed-leading-coefficient BDF in Nordsieck form, its local error test,
 * step/order selection and the modified Newton iteration.
 *
 * The preconditioner for P = I - gamma J is by default one block-Jacobi
 * sweep (exact inverse of each node's 3x3 block), as on the device.  The
 * reference's own form -- P assembled, PETSc GMRES + bjacobi/ILU(0) to
 * pc_rtol (nsim.ml:2210-2262,2419-2483) -- is restated below as well
 * (om_bdf_set_precond kind 1) so that the two can be compared: they change
 * the Krylov iteration counts, not the converged Newton corrections.
 */
#include "nmag_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define QMAXB 5
#define ETAMX1 10000.0
#define ETAMX2 10.0
#define ETAMX3 10.0
#define ETAMXF 0.2
#define ETAMIN 0.1
#define ETACF 0.25
#define ADDON 1e-6
#define BIAS1 6.0
#define BIAS2 6.0
#define BIAS3 10.0
#define ONEPSM 1.000001
#define SMALL_NST 10
#define MXNCF 10
#define MXNEF 7
#define MXNEF1 3
#define SMALL_NEF 2
#define LONG_WAIT 10
#define NLS_MAXCOR 3
#define CRDOWN 0.3
#define DGMAX 0.3
#define RDIV 2.0
#define MSBP 20
#define CORTES 0.1
#define SPILS_DGMAX 0.2
#define SPILS_MSBPRE 50
#define SPILS_DELT 0.05

struct om_bdf {
  om_state *S;
  int n, qmax, maxl;
  double rtol, atol, pc_rtol, pc_atol;
  double *zn[QMAXB + 2];
  double *ewt, *acor, *y, *tempv, *ftemp;
  double *mJ, *HJ;              /* frozen Jacobian point */
  double **V, *Hm, *givens, *yg, *work;
  double tn, h, hprime, eta, hscale, etamax, rl1, gamma, gammap, gamrat, crate, acnrm, nlscoef;
  double tau[QMAXB + 2], tq[6], l[QMAXB + 1];
  int q, qprime, qwait, L;
  long long nst, nfe, nni, nli, ncfn, netf, nsetups, npe, nps, njv, nstlp, nstlpre;
  double saved_tq5, beta0;
  double *xsol;
  int jcur, setup_done;
  double hu; int qu;
  double tstop; int tstop_set;
  struct om_ilu_pc *pc;         /* the reference's preconditioner (kind 1), or NULL */
};

static double wrms(int n, const double *x, const double *w) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) { double v = x[i] * w[i]; s += v * v; }
  return sqrt(s / n);
}

static void set_ewt(om_bdf *B, const double *y) {
  for (int i = 0; i < B->n; ++i) B->ewt[i] = 1.0 / (B->rtol * fabs(y[i]) + B->atol);
}

/* ---- the reference's preconditioner: P = I - gamma J assembled over the
 * node graph's 3x3 blocks (the reference copies its Jacobian matrix into mx,
 * scales by -gamma and adds the identity at every PC setup), solved by PETSc
 * KSP GMRES with bjacobi/ILU (nsim.ml:2210-2262,2419-2483).  On one process
 * bjacobi has one block, so the preconditioner is ILU(0) of the whole
 * matrix in natural (DOF) order.  GMRES: restarted (PETSc's default restart
 * 30), left preconditioned, zero initial guess, stopped when the estimate of
 * the preconditioned residual norm is <= max(pc_rtol * its initial value,
 * pc_atol) or after maxit iterations (the reference passes no dtol/maxit, so
 * PETSc's 10000 applies).  Restated from PETSc's documented KSPGMRES/PCILU
 * behaviour (PETSc 2.3.3 is not in the reference tree). ---- */
typedef struct om_ilu_pc {
  int n, nnz, restart, maxit;
  int *rp, *ci, *diag, *iw;
  double *a;               /* P, then its ILU(0) factors in place */
  double *a0;              /* P as assembled (matrix products) */
  double **V, *Hh, *cs, *sn, *g, *w, *res;
  long long iters;         /* GMRES iterations over the run */
} om_ilu_pc;

static void ilu_pc_free(om_ilu_pc *P) {
  if (!P) return;
  free(P->rp); free(P->ci); free(P->diag); free(P->iw); free(P->a); free(P->a0);
  if (P->V) for (int j = 0; j <= P->restart; ++j) free(P->V[j]);
  free(P->V); free(P->Hh); free(P->cs); free(P->sn); free(P->g); free(P->w); free(P->res);
  free(P);
}

/* Scalar CSR pattern of the 3x3-block matrix over the node graph (columns
 * ascending because the node columns are). */
static om_ilu_pc *ilu_pc_create(const om_mesh *M, int restart, int maxit) {
  om_ilu_pc *P = calloc(1, sizeof(om_ilu_pc));
  int N = M->n_nodes;
  P->n = 3 * N; P->restart = restart < 1 ? 30 : restart; P->maxit = maxit < 1 ? 10000 : maxit;
  P->nnz = 9 * M->nnz;
  P->rp = malloc(sizeof(int) * (P->n + 1)); P->ci = malloc(sizeof(int) * P->nnz);
  P->diag = malloc(sizeof(int) * P->n); P->iw = malloc(sizeof(int) * P->n);
  P->a = malloc(sizeof(double) * P->nnz); P->a0 = malloc(sizeof(double) * P->nnz);
  int pos = 0;
  for (int i = 0; i < N; ++i)
    for (int r = 0; r < 3; ++r) {
      int row = 3 * i + r;
      P->rp[row] = pos;
      for (int k = M->row_ptr[i]; k < M->row_ptr[i + 1]; ++k)
        for (int c = 0; c < 3; ++c) {
          int col = 3 * M->col_idx[k] + c;
          if (col == row) P->diag[row] = pos;
          P->ci[pos++] = col;
        }
    }
  P->rp[P->n] = pos;
  for (int i = 0; i < P->n; ++i) P->iw[i] = -1;
  P->V = calloc(P->restart + 1, sizeof(double *));
  for (int j = 0; j <= P->restart; ++j) P->V[j] = calloc(P->n, sizeof(double));
  P->Hh = calloc((size_t)(P->restart + 1) * P->restart, sizeof(double));
  P->cs = calloc(P->restart, sizeof(double)); P->sn = calloc(P->restart, sizeof(double));
  P->g = calloc(P->restart + 1, sizeof(double));
  P->w = calloc(P->n, sizeof(double)); P->res = calloc(P->n, sizeof(double));
  return P;
}

/* The linearised LLG right-hand side of one node (the approximate
 * Jacobian's row block, om_jv): C1 (w x H + m x hv) + C2 (w x (m x H) +
 * m x (w x H + m x hv)). */
static void llg_lin(double C1, double C2, const double *m, const double *H, const double *w, const double *hv,
                    double *out) {
  double a[3] = {w[1] * H[2] - w[2] * H[1] + (m[1] * hv[2] - m[2] * hv[1]),
                 w[2] * H[0] - w[0] * H[2] + (m[2] * hv[0] - m[0] * hv[2]),
                 w[0] * H[1] - w[1] * H[0] + (m[0] * hv[1] - m[1] * hv[0])};
  double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
  double wxH[3] = {w[1] * H[2] - w[2] * H[1], w[2] * H[0] - w[0] * H[2], w[0] * H[1] - w[1] * H[0]};
  double mxhv[3] = {m[1] * hv[2] - m[2] * hv[1], m[2] * hv[0] - m[0] * hv[2], m[0] * hv[1] - m[1] * hv[0]};
  double t1[3] = {w[1] * mxH[2] - w[2] * mxH[1], w[2] * mxH[0] - w[0] * mxH[2], w[0] * mxH[1] - w[1] * mxH[0]};
  double u[3] = {wxH[0] + mxhv[0], wxH[1] + mxhv[1], wxH[2] + mxhv[2]};
  double t2[3] = {m[1] * u[2] - m[2] * u[1], m[2] * u[0] - m[0] * u[2], m[0] * u[1] - m[1] * u[0]};
  for (int d = 0; d < 3; ++d) out[d] = C1 * a[d] + C2 * (t1[d] + t2[d]);
}

/* P = I - gamma J(mJ, HJ) into a0 and a (blocks probed column by column
 * through the node's linearisation: exact, since it is linear in w, hv). */
static void ilu_pc_assemble(om_ilu_pc *P, const om_state *S, const double *mJ, const double *HJ, double gamma) {
  const om_mesh *M = S->M;
  const double c = S->mat.exch_coeff, C1 = S->mat.C1, C2 = S->mat.C2;
  for (int i = 0; i < M->n_nodes; ++i) {
    const double *m = mJ + 3 * (size_t)i, *H = HJ + 3 * (size_t)i;
    const double pin = S->pin ? S->pin[i] : 1.0;
    const int deg = M->row_ptr[i + 1] - M->row_ptr[i];
    for (int q = 0; q < deg; ++q) {
      const int k = M->row_ptr[i] + q, j = M->col_idx[k];
      const double kap = -c * M->K[k] / M->vol[i];
      for (int cc = 0; cc < 3; ++cc) {
        double w[3] = {0, 0, 0}, hv[3] = {0, 0, 0}, col[3];
        hv[cc] = kap;
        if (j == i) w[cc] = 1.0;
        llg_lin(C1, C2, m, H, w, hv, col);
        for (int r = 0; r < 3; ++r) {
          const int at = P->rp[3 * i + r] + 3 * q + cc;
          P->a0[at] = (j == i && r == cc ? 1.0 : 0.0) - gamma * (pin * col[r]);
        }
      }
    }
  }
  memcpy(P->a, P->a0, sizeof(double) * P->nnz);
}

/* ILU(0) in place (row-wise IKJ form); 0, or -1 on a zero pivot. */
static int ilu_pc_factor(om_ilu_pc *P) {
  int *iw = P->iw;
  double *a = P->a;
  for (int i = 0; i < P->n; ++i) {
    for (int p = P->rp[i]; p < P->rp[i + 1]; ++p) iw[P->ci[p]] = p;
    for (int p = P->rp[i]; p < P->rp[i + 1] && P->ci[p] < i; ++p) {
      const int k = P->ci[p];
      const double piv = a[P->diag[k]];
      if (piv == 0.0) return -1;
      const double lik = a[p] / piv;
      a[p] = lik;
      for (int q = P->diag[k] + 1; q < P->rp[k + 1]; ++q) {
        const int at = iw[P->ci[q]];
        if (at >= 0) a[at] -= lik * a[q];
      }
    }
    for (int p = P->rp[i]; p < P->rp[i + 1]; ++p) iw[P->ci[p]] = -1;
    if (a[P->diag[i]] == 0.0) return -1;
  }
  return 0;
}

/* z = (LU)^{-1} r (unit lower L, upper U with the diagonal). */
static void ilu_pc_subst(const om_ilu_pc *P, const double *r, double *z) {
  for (int i = 0; i < P->n; ++i) {
    double s = r[i];
    for (int p = P->rp[i]; p < P->diag[i]; ++p) s -= P->a[p] * z[P->ci[p]];
    z[i] = s;
  }
  for (int i = P->n - 1; i >= 0; --i) {
    double s = z[i];
    for (int p = P->diag[i] + 1; p < P->rp[i + 1]; ++p) s -= P->a[p] * z[P->ci[p]];
    z[i] = s / P->a[P->diag[i]];
  }
}

static void ilu_pc_matvec(const om_ilu_pc *P, const double *v, double *out) {
  for (int i = 0; i < P->n; ++i) {
    double s = 0.0;
    for (int p = P->rp[i]; p < P->rp[i + 1]; ++p) s += P->a0[p] * v[P->ci[p]];
    out[i] = s;
  }
}

/* GMRES(restart) on P z = r, left-preconditioned by the ILU(0) factors. */
static void ilu_pc_solve(om_ilu_pc *P, const double *r, double *z, double rtol, double atol) {
  const int n = P->n, mr = P->restart;
  double **V = P->V, *g = P->g, *w = P->w;
#define HH(i, j) P->Hh[(size_t)(i) * mr + (j)]
  memset(z, 0, sizeof(double) * n);
  double tol = -1.0;
  int it = 0;
  for (;;) {
    /* preconditioned residual of the current iterate */
    if (it == 0) memcpy(P->res, r, sizeof(double) * n);
    else {
      ilu_pc_matvec(P, z, w);
      for (int i = 0; i < n; ++i) P->res[i] = r[i] - w[i];
    }
    ilu_pc_subst(P, P->res, V[0]);
    double beta = 0.0;
    for (int i = 0; i < n; ++i) beta += V[0][i] * V[0][i];
    beta = sqrt(beta);
    if (tol < 0.0) tol = fmax(rtol * beta, atol);
    if (beta <= tol || beta == 0.0 || it >= P->maxit) break;
    for (int i = 0; i < n; ++i) V[0][i] /= beta;
    memset(g, 0, sizeof(double) * (mr + 1));
    g[0] = beta;
    int kdim = 0;
    double resid = beta;
    for (int j = 0; j < mr && it < P->maxit; ++j) {
      ilu_pc_matvec(P, V[j], P->res);
      ilu_pc_subst(P, P->res, w);
      ++it;
      for (int k = 0; k <= j; ++k) {   /* modified Gram-Schmidt */
        double h = 0.0;
        for (int i = 0; i < n; ++i) h += V[k][i] * w[i];
        HH(k, j) = h;
        for (int i = 0; i < n; ++i) w[i] -= h * V[k][i];
      }
      double hn = 0.0;
      for (int i = 0; i < n; ++i) hn += w[i] * w[i];
      hn = sqrt(hn);
      HH(j + 1, j) = hn;
      for (int k = 0; k < j; ++k) {
        const double t1 = HH(k, j), t2 = HH(k + 1, j);
        HH(k, j) = P->cs[k] * t1 + P->sn[k] * t2;
        HH(k + 1, j) = -P->sn[k] * t1 + P->cs[k] * t2;
      }
      const double aa = HH(j, j), bb = HH(j + 1, j), den = hypot(aa, bb);
      P->cs[j] = den == 0.0 ? 1.0 : aa / den;
      P->sn[j] = den == 0.0 ? 0.0 : bb / den;
      HH(j, j) = den; HH(j + 1, j) = 0.0;
      g[j + 1] = -P->sn[j] * g[j];
      g[j] = P->cs[j] * g[j];
      resid = fabs(g[j + 1]);
      kdim = j + 1;
      if (resid <= tol || hn == 0.0) break;
      for (int i = 0; i < n; ++i) V[j + 1][i] = w[i] / hn;
    }
    for (int k = kdim - 1; k >= 0; --k) {   /* y = H^{-1} g, then z += V y */
      double s = g[k];
      for (int jj = k + 1; jj < kdim; ++jj) s -= HH(k, jj) * g[jj];
      g[k] = s / HH(k, k);
    }
    for (int k = 0; k < kdim; ++k) for (int i = 0; i < n; ++i) z[i] += g[k] * V[k][i];
    if (resid <= tol || it >= P->maxit) break;
  }
  P->iters += it;
#undef HH
}

void om_bdf_set_precond(om_bdf *B, int kind, int restart, int maxit) {
  ilu_pc_free(B->pc);
  B->pc = kind == 1 ? ilu_pc_create(B->S->M, restart, maxit) : NULL;
}

long long om_bdf_pc_iterations(const om_bdf *B) { return B->pc ? B->pc->iters : 0; }

void om_pc_matrix_apply(const om_state *S, const double *mJ, const double *HJ, double gamma, const double *v,
                        double *out) {
  om_ilu_pc *P = ilu_pc_create(S->M, 1, 1);
  ilu_pc_assemble(P, S, mJ, HJ, gamma);
  ilu_pc_matvec(P, v, out);
  ilu_pc_free(P);
}

om_bdf *om_bdf_create(om_state *S, int qmax, int maxl, double rtol, double atol, double pc_rtol, double pc_atol) {
  om_bdf *B = calloc(1, sizeof(om_bdf));
  B->S = S; B->n = 3 * S->M->n_nodes;
  B->qmax = qmax < 1 ? 1 : (qmax > QMAXB ? QMAXB : qmax);
  B->maxl = maxl < 1 ? 5 : maxl;
  B->rtol = rtol; B->atol = atol; B->pc_rtol = pc_rtol; B->pc_atol = pc_atol;
  int n = B->n;
  for (int j = 0; j <= B->qmax + 1; ++j) B->zn[j] = calloc(n, sizeof(double));
  B->ewt = calloc(n, sizeof(double)); B->acor = calloc(n, sizeof(double)); B->y = calloc(n, sizeof(double));
  B->tempv = calloc(n, sizeof(double)); B->ftemp = calloc(n, sizeof(double));
  B->mJ = calloc(n, sizeof(double)); B->HJ = calloc(n, sizeof(double));
  B->V = calloc(B->maxl + 1, sizeof(double *));
  for (int j = 0; j <= B->maxl; ++j) B->V[j] = calloc(n, sizeof(double));
  B->Hm = calloc((size_t)(B->maxl + 1) * B->maxl, sizeof(double));
  B->givens = calloc(2 * (size_t)B->maxl, sizeof(double));
  B->yg = calloc(B->maxl + 1, sizeof(double));
  B->work = calloc(n, sizeof(double));
  B->xsol = calloc(n, sizeof(double));
  return B;
}

void om_bdf_free(om_bdf *B) {
  if (!B) return;
  for (int j = 0; j <= B->qmax + 1; ++j) free(B->zn[j]);
  free(B->ewt); free(B->acor); free(B->y); free(B->tempv); free(B->ftemp); free(B->mJ); free(B->HJ);
  for (int j = 0; j <= B->maxl; ++j) free(B->V[j]);
  free(B->V); free(B->Hm); free(B->givens); free(B->yg); free(B->work); free(B->xsol);
  ilu_pc_free(B->pc);
  free(B);
}

static int rhs(om_bdf *B, const double *y, double *f) {
  B->nfe++;
  return om_rhs(B->S, y, f);
}

/* Initial step size (cvHin / cvUpperBoundH0 / cvYddNorm of CVODE): geometric
 * mean of a lower bound 100*uround*max(|t0|,|tout|) and an upper bound
 * min(0.1*|tout-t0|, 1/max_i(|y'_i| / (0.1|y_i| + rtol|y_i| + atol))), refined
 * by up to 4 estimates of ||y''|| from a forward-Euler difference, biased 0.5. */
static double initial_h(om_bdf *B, double tout) {
  int n = B->n;
  double tdist = fabs(tout - B->tn);
  double tround = DBL_EPSILON * (fabs(B->tn) > fabs(tout) ? fabs(B->tn) : fabs(tout));
  double hlb = 100.0 * tround;
  double hub_inv = 0.0;
  for (int i = 0; i < n; ++i) {
    double den = 0.1 * fabs(B->zn[0][i]) + 1.0 / B->ewt[i];
    double v = fabs(B->zn[1][i]) / den;
    if (v > hub_inv) hub_inv = v;
  }
  double hub = 0.1 * tdist;
  if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
  double hg = sqrt(hlb * hub);
  if (hub < hlb) return hg;
  double hnew = hg;
  int count = 0;
  for (;;) {
    for (int i = 0; i < n; ++i) B->y[i] = hg * B->zn[1][i] + B->zn[0][i];
    if (rhs(B, B->y, B->tempv)) return hg;
    for (int i = 0; i < n; ++i) B->tempv[i] = (B->tempv[i] - B->zn[1][i]) * (1.0 / hg);
    double yddnrm = wrms(n, B->tempv, B->ewt);
    hnew = (yddnrm * hub * hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(hg * hub);
    count++;
    if (count >= 4) break;
    double hrat = hnew / hg;
    if (hrat > 0.5 && hrat < 2.0) break;
    if (count >= 2 && hrat > 2.0) { hnew = hg; break; }
    hg = hnew;
  }
  double h0 = 0.5 * hnew;
  if (h0 < hlb) h0 = hlb;
  if (h0 > hub) h0 = hub;
  return h0;
}

int om_bdf_init(om_bdf *B, double t0, const double *m0) {
  B->tn = t0; B->q = 1; B->L = 2; B->qwait = B->L;
  B->nst = B->nfe = B->nni = B->nli = B->ncfn = B->netf = B->nsetups = B->npe = B->nps = B->njv = 0;
  B->nstlp = B->nstlpre = 0;
  B->etamax = ETAMX1; B->h = 0.0; B->hu = 0.0; B->qu = 0;
  B->nlscoef = CORTES;
  B->setup_done = 0; B->jcur = 0;
  memcpy(B->zn[0], m0, sizeof(double) * B->n);
  for (int j = 1; j <= B->qmax + 1; ++j) memset(B->zn[j], 0, sizeof(double) * B->n);
  for (int i = 0; i <= QMAXB + 1; ++i) B->tau[i] = 0.0;
  for (int i = 0; i < 6; ++i) B->tq[i] = 0.0;
  set_ewt(B, m0);
  if (rhs(B, B->zn[0], B->zn[1])) return 1;
  return 0;
}

/* ---- preconditioner: P = I - gamma J, one exact 3x3 block-Jacobi sweep ---- */
static void block_of_J(const om_bdf *B, int i, double Jb[3][3]) {
  const om_state *S = B->S;
  const om_mesh *M = S->M;
  int pos = M->row_ptr[i];
  while (M->col_idx[pos] != i) ++pos;
  double kap = -S->mat.exch_coeff * M->K[pos] / M->vol[i];
  const double *m = B->mJ + 3 * i, *H = B->HJ + 3 * i;
  double C1 = S->mat.C1, C2 = S->mat.C2;
  for (int c = 0; c < 3; ++c) {
    double w[3] = {0, 0, 0}; w[c] = 1.0;
    double hv[3] = {kap * w[0], kap * w[1], kap * w[2]};
    double a[3] = {w[1] * H[2] - w[2] * H[1] + (m[1] * hv[2] - m[2] * hv[1]),
                   w[2] * H[0] - w[0] * H[2] + (m[2] * hv[0] - m[0] * hv[2]),
                   w[0] * H[1] - w[1] * H[0] + (m[0] * hv[1] - m[1] * hv[0])};
    double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
    double wxH[3] = {w[1] * H[2] - w[2] * H[1], w[2] * H[0] - w[0] * H[2], w[0] * H[1] - w[1] * H[0]};
    double mxhv[3] = {m[1] * hv[2] - m[2] * hv[1], m[2] * hv[0] - m[0] * hv[2], m[0] * hv[1] - m[1] * hv[0]};
    double t1[3] = {w[1] * mxH[2] - w[2] * mxH[1], w[2] * mxH[0] - w[0] * mxH[2], w[0] * mxH[1] - w[1] * mxH[0]};
    double u[3] = {wxH[0] + mxhv[0], wxH[1] + mxhv[1], wxH[2] + mxhv[2]};
    double t2[3] = {m[1] * u[2] - m[2] * u[1], m[2] * u[0] - m[0] * u[2], m[0] * u[1] - m[1] * u[0]};
    for (int d = 0; d < 3; ++d) Jb[d][c] = C1 * a[d] + C2 * (t1[d] + t2[d]);
  }
  if (S->pin) /* the Jacobian rows carry the pin factor (nmag_lam.py:432-436) */
    for (int d = 0; d < 3; ++d) for (int c = 0; c < 3; ++c) Jb[d][c] *= S->pin[i];
}

static void psolve(om_bdf *B, const double *r, double *z) {
  if (B->pc) {   /* the reference's form: GMRES + ILU(0) on the assembled P */
    ilu_pc_solve(B->pc, r, z, B->pc_rtol, B->pc_atol);
    B->nps++;
    return;
  }
  int N = B->S->M->n_nodes;
  double g = B->gammap; /* P = I - gamma J was built at the last setup */
  for (int i = 0; i < N; ++i) {
    double Jb[3][3], P[3][3];
    block_of_J(B, i, Jb);
    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) P[a][b] = (a == b ? 1.0 : 0.0) - g * Jb[a][b];
    double c00 = P[1][1] * P[2][2] - P[1][2] * P[2][1];
    double c01 = P[1][2] * P[2][0] - P[1][0] * P[2][2];
    double c02 = P[1][0] * P[2][1] - P[1][1] * P[2][0];
    double det = P[0][0] * c00 + P[0][1] * c01 + P[0][2] * c02;
    double inv = 1.0 / det;
    const double *ri = r + 3 * i;
    double Pi[3][3] = {{c00 * inv, (P[0][2] * P[2][1] - P[0][1] * P[2][2]) * inv, (P[0][1] * P[1][2] - P[0][2] * P[1][1]) * inv},
                       {c01 * inv, (P[0][0] * P[2][2] - P[0][2] * P[2][0]) * inv, (P[0][2] * P[1][0] - P[0][0] * P[1][2]) * inv},
                       {c02 * inv, (P[0][1] * P[2][0] - P[0][0] * P[2][1]) * inv, (P[0][0] * P[1][1] - P[0][1] * P[1][0]) * inv}};
    for (int a = 0; a < 3; ++a) z[3 * i + a] = (Pi[a][0] * ri[0] + Pi[a][1] * ri[1]) + Pi[a][2] * ri[2];
  }
  B->nps++;
}

/* psetup: if !jok, re-evaluate the RHS at y to get H_total and freeze (m, H)
 * as the Jacobian point (nsim.ml:2315-2398 re-Jacobi); returns jcur. */
static int psetup(om_bdf *B, int jok, const double *ypred) {
  B->npe++;
  int jcur = 0;
  if (!jok) {
    /* f(ypred) was evaluated just before by the Newton driver, so S->h_total
       is the field at ypred (the reference re-runs the RHS, nsim.ml:2338-2348). */
    memcpy(B->mJ, ypred, sizeof(double) * B->n);
    memcpy(B->HJ, B->S->h_total, sizeof(double) * B->n);
    jcur = 1;
  }
  if (B->pc) {   /* the reference rebuilds I - gamma J at every setup (nsim.ml:2440-2452) */
    ilu_pc_assemble(B->pc, B->S, B->mJ, B->HJ, B->gamma);
    if (ilu_pc_factor(B->pc)) return -1;
  }
  return jcur;
}

/* SPGMR with left preconditioning, scaling by ewt, modified Gram-Schmidt,
 * no restarts.  Solves (I - gamma J) x = b to ||ewt . P^{-1}(b - A x)||_2 <= delta. */
static int spgmr(om_bdf *B, const double *b, double *x, double delta, int *nli_out) {
  int n = B->n, maxl = B->maxl;
  double **V = B->V, *Hm = B->Hm, *gv = B->givens, *yg = B->yg, *w = B->work;
#define HM(i, j) Hm[(size_t)(i) * maxl + (j)]
  memset(x, 0, sizeof(double) * n);
  psolve(B, b, w);
  for (int i = 0; i < n; ++i) V[0][i] = B->ewt[i] * w[i];
  double rho = 0.0; for (int i = 0; i < n; ++i) rho += V[0][i] * V[0][i];
  rho = sqrt(rho);
  *nli_out = 0;
  if (rho <= delta) return 0;
  B->beta0 = rho;
  for (int i = 0; i < n; ++i) V[0][i] /= rho;
  yg[0] = rho;
  int l, converged = 0, kdim = 0;
  for (l = 0; l < maxl; ++l) {
    /* w = A V[l]/ewt, then P^{-1} */
    for (int i = 0; i < n; ++i) B->tempv[i] = V[l][i] / B->ewt[i];
    om_jv(B->S, B->mJ, B->HJ, B->tempv, w);
    B->njv++;
    for (int i = 0; i < n; ++i) w[i] = B->tempv[i] - B->gamma * w[i];
    psolve(B, w, B->tempv);
    for (int i = 0; i < n; ++i) V[l + 1][i] = B->ewt[i] * B->tempv[i];
    for (int k = 0; k <= l; ++k) {
      double hk = 0.0; for (int i = 0; i < n; ++i) hk += V[k][i] * V[l + 1][i];
      HM(k, l) = hk;
      for (int i = 0; i < n; ++i) V[l + 1][i] -= hk * V[k][i];
    }
    double hn = 0.0; for (int i = 0; i < n; ++i) hn += V[l + 1][i] * V[l + 1][i];
    hn = sqrt(hn);
    HM(l + 1, l) = hn;
    /* apply previous Givens rotations, then a new one */
    for (int k = 0; k < l; ++k) {
      double c = gv[2 * k], s = gv[2 * k + 1];
      double t1 = HM(k, l), t2 = HM(k + 1, l);
      HM(k, l) = c * t1 - s * t2; HM(k + 1, l) = s * t1 + c * t2;
    }
    double a = HM(l, l), bb = HM(l + 1, l), c, s;
    if (bb == 0.0) { c = 1.0; s = 0.0; }
    else if (fabs(bb) > fabs(a)) { double t = a / bb; s = -1.0 / sqrt(1.0 + t * t); c = -s * t; }
    else { double t = bb / a; c = 1.0 / sqrt(1.0 + t * t); s = -c * t; }
    gv[2 * l] = c; gv[2 * l + 1] = s;
    HM(l, l) = c * a - s * bb; HM(l + 1, l) = 0.0;
    yg[l + 1] = s * yg[l]; yg[l] = c * yg[l];
    rho = fabs(yg[l + 1]);
    kdim = l + 1;
    if (rho <= delta) { converged = 1; break; }
    if (hn == 0.0) break;
    for (int i = 0; i < n; ++i) V[l + 1][i] /= hn;
  }
  *nli_out = kdim;
  /* back substitution */
  for (int k = kdim - 1; k >= 0; --k) {
    double sum = yg[k];
    for (int j = k + 1; j < kdim; ++j) sum -= HM(k, j) * yg[j];
    yg[k] = sum / HM(k, k);
  }
  for (int k = 0; k < kdim; ++k) for (int i = 0; i < n; ++i) x[i] += yg[k] * V[k][i];
  for (int i = 0; i < n; ++i) x[i] /= B->ewt[i];
#undef HM
  /* 0 converged, 2 residual reduced but not converged, 1 failure */
  if (converged) return 0;
  return (rho < B->beta0) ? 2 : 1;
}

/* ---- Nordsieck array operations ---- */
static void predict(om_bdf *B) {
  B->tn += B->h;
  for (int k = 1; k <= B->q; ++k)
    for (int j = B->q; j >= k; --j)
      for (int i = 0; i < B->n; ++i) B->zn[j - 1][i] += B->zn[j][i];
}

static void restore(om_bdf *B, double saved_t) {
  B->tn = saved_t;
  for (int k = 1; k <= B->q; ++k)
    for (int j = B->q; j >= k; --j)
      for (int i = 0; i < B->n; ++i) B->zn[j - 1][i] -= B->zn[j][i];
}

static void rescale(om_bdf *B) {
  double factor = B->eta;
  for (int j = 1; j <= B->q; ++j) {
    for (int i = 0; i < B->n; ++i) B->zn[j][i] *= factor;
    factor *= B->eta;
  }
  B->h = B->hscale * B->eta;
  B->hprime = B->h;
  B->hscale = B->h;
}

/* BDF coefficients l[] and test quantities tq[] for the current h, q and
 * step history tau[] (fixed-leading-coefficient form). */
static void set_bdf(om_bdf *B) {
  int q = B->q;
  double *l = B->l, *tau = B->tau, h = B->h;
  double alpha0, alpha0_hat, xi_inv, xistar_inv, hsum;
  l[0] = l[1] = xi_inv = xistar_inv = 1.0;
  for (int i = 2; i <= QMAXB; ++i) l[i] = 0.0;
  alpha0 = alpha0_hat = -1.0;
  hsum = h;
  if (q > 1) {
    for (int j = 2; j < q; ++j) {
      hsum += tau[j - 1];
      xi_inv = h / hsum;
      alpha0 -= 1.0 / j;
      for (int i = j; i >= 1; --i) l[i] += l[i - 1] * xi_inv;
    }
    alpha0 -= 1.0 / q;
    xistar_inv = -l[1] - alpha0;
    hsum += tau[q - 1];
    xi_inv = h / hsum;
    alpha0_hat = -l[1] - xi_inv;
    for (int i = q; i >= 1; --i) l[i] += l[i - 1] * xistar_inv;
  }
  double A1 = 1.0 - alpha0_hat + alpha0;
  double A2 = 1.0 + q * A1;
  B->tq[2] = fabs(A1 / (alpha0 * A2));
  B->tq[5] = fabs(A2 * xistar_inv / (l[q] * xi_inv));
  if (B->qwait == 1) {
    if (q > 1) {
      double C = xistar_inv / l[q];
      double A3 = alpha0 + 1.0 / q;
      double A4 = alpha0_hat + xi_inv;
      double Cpinv = (1.0 - A4 + A3) / A3;
      B->tq[1] = fabs(C * Cpinv);
    } else B->tq[1] = 1.0;
    hsum += tau[q];
    xi_inv = h / hsum;
    double A5 = alpha0 - 1.0 / (q + 1);
    double A6 = alpha0_hat - xi_inv;
    double Cppinv = (1.0 - A6 + A5) / A2;
    B->tq[3] = fabs(Cppinv / (xi_inv * (q + 2) * A5));
  }
  B->tq[4] = B->nlscoef / B->tq[2];
}

/* Newton iteration on G(y) = y - ypred - gamma (f(y) - ...), returns
 * 0 ok, 1 recoverable convergence failure, <0 unrecoverable. */
static int nls(om_bdf *B, int nflag_first) {
  int n = B->n;
  int convfail_bad_j = 0;
  int call_setup = (nflag_first == 2 /* prev conv fail */) || (nflag_first == 3 /* prev err fail */) ||
                   (B->nst == 0) || (B->nst >= B->nstlp + MSBP) || (fabs(B->gamrat - 1.0) > DGMAX);
  int convfail_other = !(nflag_first == 1 || nflag_first == 3); /* FIRST_CALL or PREV_ERR_FAIL -> NO_FAILURES */
  for (;;) {
    if (rhs(B, B->zn[0], B->ftemp)) return -2;
    if (call_setup) {
      double dgamma = fabs(B->gamma / B->gammap - 1.0);
      int jbad = (B->nst == 0) || (B->nst > B->nstlpre + SPILS_MSBPRE) ||
                 (convfail_bad_j && dgamma < SPILS_DGMAX) || (!convfail_bad_j && convfail_other);
      if (!B->setup_done) jbad = 1;
      int jc = psetup(B, !jbad, B->zn[0]);
      if (jc < 0) return -3;
      B->jcur = jc;
      if (jc) B->nstlpre = B->nst;
      B->setup_done = 1;
      B->nsetups++;
      B->crate = 1.0; B->gammap = B->gamma; B->nstlp = B->nst; B->gamrat = 1.0;
    }
    memset(B->acor, 0, sizeof(double) * n);
    memcpy(B->y, B->zn[0], sizeof(double) * n);
    int m = 0;
    double delp = 0.0, del;
    int retry = 0;
    for (;;) {
      B->nni++;
      for (int i = 0; i < n; ++i) B->tempv[i] = B->gamma * B->ftemp[i] - (B->rl1 * B->zn[1][i] + B->acor[i]);
      /* linear solve (CVSpgmrSolve): skip when ||b|| is already below
         delt*tq[4]; SPGMR tolerance delta = delt*tq[4]*sqrt(n) on the
         scaled 2-norm; no gamma-ratio rescaling since Atimes uses the
         current gamma. */
      double deltar = SPILS_DELT * B->tq[4];
      double bnorm = wrms(n, B->tempv, B->ewt);
      int lflag = 0;
      if (bnorm <= deltar) {
        if (m > 0) memset(B->tempv, 0, sizeof(double) * n);
      } else {
        int nli = 0;
        int sr = spgmr(B, B->tempv, B->xsol, deltar * sqrt((double)n), &nli);
        B->nli += nli;
        memcpy(B->tempv, B->xsol, sizeof(double) * n);
        if (sr == 1 || (sr == 2 && m > 0)) lflag = 1;
      }
      if (lflag) {
        if (!B->jcur) { convfail_bad_j = 1; call_setup = 1; retry = 1; }
        break;
      }
      del = wrms(n, B->tempv, B->ewt);
      for (int i = 0; i < n; ++i) { B->acor[i] += B->tempv[i]; B->y[i] = B->zn[0][i] + B->acor[i]; }
      if (m > 0) { double r = del / delp; B->crate = CRDOWN * B->crate > r ? CRDOWN * B->crate : r; }
      double dcon = del * (B->crate < 1.0 ? B->crate : 1.0) / B->tq[4];
      if (dcon <= 1.0) {
        B->acnrm = (m == 0) ? del : wrms(n, B->acor, B->ewt);
        B->jcur = 0;
        return 0;
      }
      ++m;
      if (m == NLS_MAXCOR || (m >= 2 && del > RDIV * delp)) {
        if (!B->jcur) { convfail_bad_j = 1; call_setup = 1; retry = 1; }
        break;
      }
      delp = del;
      if (rhs(B, B->y, B->ftemp)) return -2;
    }
    if (!retry) return 1;
  }
}

static void complete_step(om_bdf *B) {
  B->nst++;
  B->hu = B->h; B->qu = B->q;
  for (int i = B->q; i >= 2; --i) B->tau[i] = B->tau[i - 1];
  if (B->q == 1 && B->nst > 1) B->tau[2] = B->tau[1];
  B->tau[1] = B->h;
  for (int j = 0; j <= B->q; ++j)
    for (int i = 0; i < B->n; ++i) B->zn[j][i] += B->l[j] * B->acor[i];
  B->qwait--;
  if (B->qwait == 1 && B->q != B->qmax) {
    memcpy(B->zn[B->qmax], B->acor, sizeof(double) * B->n);
    B->saved_tq5 = B->tq[5];
  }
}

static void adjust_order(om_bdf *B, int deltaq) {
  /* BDF order change of the Nordsieck array (cvAdjustBDF) */
  int q = B->q, n = B->n;
  if (deltaq == 1) {
    /* increase: zn[q+1] = (l-style) correction from saved acor (cvIncreaseBDF) */
    double *l = B->l;
    for (int i = 0; i <= B->qmax; ++i) l[i] = 0.0;
    l[2] = 1.0;
    double alpha0 = -1.0, alpha1 = 1.0, prod = 1.0, xiold = 1.0, hsum = B->hscale;
    if (q > 1) {
      for (int j = 1; j < q; ++j) {
        hsum += B->tau[j + 1];
        double xi = hsum / B->hscale;
        prod *= xi;
        alpha0 -= 1.0 / (j + 1);
        alpha1 += 1.0 / xi;
        for (int i = j + 2; i >= 2; --i) l[i] = l[i] * xiold + l[i - 1];
        xiold = xi;
      }
    }
    double A1 = (-alpha0 - alpha1) / prod;
    for (int i = 0; i < n; ++i) B->zn[q + 1][i] = A1 * B->zn[B->qmax][i];
    for (int j = 2; j <= q; ++j)
      for (int i = 0; i < n; ++i) B->zn[j][i] += l[j] * B->zn[q + 1][i];
  } else if (deltaq == -1) {
    /* decrease (cvDecreaseBDF) */
    double *l = B->l;
    for (int i = 0; i <= B->qmax; ++i) l[i] = 0.0;
    l[2] = 1.0;
    double hsum = 0.0;
    for (int j = 1; j <= q - 2; ++j) {
      hsum += B->tau[j];
      double xi = hsum / B->hscale;
      for (int i = j + 2; i >= 2; --i) l[i] = l[i] * xi + l[i - 1];
    }
    for (int j = 2; j < q; ++j)
      for (int i = 0; i < n; ++i) B->zn[j][i] -= l[j] * B->zn[q][i];
  }
}

static void prepare_next_step(om_bdf *B, double dsm) {
  if (B->etamax == 1.0) { B->qwait = B->qwait > 2 ? B->qwait : 2; B->qprime = B->q; B->hprime = B->h; B->eta = 1.0; return; }
  double etaq = 1.0 / (pow(BIAS2 * dsm, 1.0 / B->L) + ADDON);
  if (B->qwait != 0) {
    B->eta = etaq; B->qprime = B->q;
  } else {
    B->qwait = 2;
    double etaqm1 = 0.0, etaqp1 = 0.0;
    if (B->q > 1) {
      double ddn = wrms(B->n, B->zn[B->q], B->ewt) * B->tq[1];
      etaqm1 = 1.0 / (pow(BIAS1 * ddn, 1.0 / B->q) + ADDON);
    }
    if (B->q != B->qmax && B->saved_tq5 != 0.0) {
      double cquot = (B->tq[5] / B->saved_tq5) * pow(B->h / B->tau[2], (double)B->L);
      for (int i = 0; i < B->n; ++i) B->tempv[i] = B->acor[i] - cquot * B->zn[B->qmax][i];
      double dup = wrms(B->n, B->tempv, B->ewt) * B->tq[3];
      etaqp1 = 1.0 / (pow(BIAS3 * dup, 1.0 / (B->L + 1)) + ADDON);
    }
    /* choose the order with the largest eta */
    if (etaqm1 > etaq && etaqm1 >= etaqp1) { B->eta = etaqm1; B->qprime = B->q - 1; }
    else if (etaqp1 > etaq) { B->eta = etaqp1; B->qprime = B->q + 1; memcpy(B->zn[B->qmax], B->acor, sizeof(double) * B->n); }
    else { B->eta = etaq; B->qprime = B->q; }
  }
  if (B->eta < 1.5) { B->eta = 1.0; B->qprime = B->q; }   /* THRESH: keep h unless it can grow by 1.5 */
  else if (B->eta > B->etamax) B->eta = B->etamax;
  B->etamax = (B->nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
  B->hprime = B->h * B->eta;
  if (B->qprime < B->q) B->qwait = B->L > 2 ? B->L : 2;
}

/* One internal step (cvStep).  Returns 0 ok, >0 failure. */
static int step(om_bdf *B) {
  double saved_t = B->tn;
  int ncf = 0, nef = 0;
  int nflag = 1; /* FIRST_CALL */
  if (B->nst > 0 && (B->hprime != B->h || B->qprime != B->q)) {
    /* adjust order and step size */
    if (B->qprime != B->q) {
      int dq = B->qprime - B->q;
      B->hscale = B->h;
      adjust_order(B, dq);
      B->q = B->qprime; B->L = B->q + 1; B->qwait = B->L;
    }
    B->hscale = B->h;
    B->eta = B->hprime / B->h;
    rescale(B);
  }
  for (;;) {
    predict(B);
    set_bdf(B);
    B->rl1 = 1.0 / B->l[1];
    B->gamma = B->h * B->rl1;
    if (B->nst == 0) B->gammap = B->gamma;
    B->gamrat = (B->nst > 0) ? B->gamma / B->gammap : 1.0;
    int r = nls(B, nflag);
    if (r < 0) { restore(B, saved_t); return 10 - r; }
    if (r == 1) {
      /* convergence failure: shrink h and retry */
      B->ncfn++; ncf++;
      restore(B, saved_t);
      if (ncf == MXNCF) return 4;
      B->etamax = 1.0;
      B->eta = ETACF;
      B->hscale = B->h;
      rescale(B);
      nflag = 2;
      continue;
    }
    double dsm = B->acnrm * B->tq[2];
    if (dsm <= 1.0) {
      complete_step(B);
      prepare_next_step(B, dsm);
      B->etamax = (B->nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
      /* scale the Nordsieck history for a step-size-only change at the next call */
      return 0;
    }
    /* error test failure */
    B->netf++; nef++;
    restore(B, saved_t);
    if (nef == MXNEF) return 5;
    B->etamax = 1.0;
    if (nef <= MXNEF1) {
      B->eta = 1.0 / (pow(BIAS2 * dsm, 1.0 / B->L) + ADDON);
      if (B->eta < ETAMIN) B->eta = ETAMIN;
      if (nef >= SMALL_NEF && B->eta > ETAMXF) B->eta = ETAMXF;
      B->hscale = B->h;
      rescale(B);
    } else if (B->q > 1) {
      /* after MXNEF1 failures: force an order reduction */
      B->eta = ETAMIN;
      B->hscale = B->h;
      adjust_order(B, -1);
      B->L = B->q; B->q--; B->qwait = B->L;
      rescale(B);
    } else {
      /* already order 1: restart from y with a fresh derivative */
      B->eta = ETAMIN;
      B->h *= B->eta; B->hscale = B->h; B->hprime = B->h;
      B->qwait = LONG_WAIT;
      if (rhs(B, B->zn[0], B->tempv)) return 12;
      for (int i = 0; i < B->n; ++i) B->zn[1][i] = B->h * B->tempv[i];
    }
    nflag = 3; /* PREV_ERR_FAIL */
  }
}

/* Dense output: y(t) from the Nordsieck array (CVodeGetDky, k = 0). */
static void interpolate(const om_bdf *B, double t, double *out) {
  double s = (t - B->tn) / B->h;
  int q = B->q;
  for (int i = 0; i < B->n; ++i) {
    double v = B->zn[q][i];
    for (int j = q - 1; j >= 0; --j) v = B->zn[j][i] + s * v;
    out[i] = v;
  }
}

int om_bdf_advance(om_bdf *B, double tout, int exact_tstop, long long max_steps, double *t_reached, double *m_out) {
  B->tstop_set = exact_tstop; B->tstop = tout;
  if (B->nst == 0 && B->h == 0.0) {
    double h0 = initial_h(B, tout);
    if (exact_tstop && (B->tn + h0 - tout) * (tout - B->tn) > 0.0) h0 = (tout - B->tn) * (1.0 - 4.0 * DBL_EPSILON);
    B->h = h0; B->hprime = h0; B->hscale = h0; B->qprime = B->q;
    for (int i = 0; i < B->n; ++i) B->zn[1][i] *= h0;
  }
  long long taken = 0;
  double troundoff = 100.0 * DBL_EPSILON * (fabs(B->tn) + fabs(B->h));
  /* already past tout with interpolation possible */
  for (;;) {
    if (!exact_tstop && (B->tn - tout) * B->h >= 0.0) { interpolate(B, tout, m_out); *t_reached = tout; return 0; }
    if (exact_tstop && fabs(B->tn - tout) <= troundoff) { interpolate(B, tout, m_out); *t_reached = tout; return 0; }
    if (max_steps >= 0 && taken >= max_steps) { memcpy(m_out, B->zn[0], sizeof(double) * B->n); *t_reached = B->tn; return 0; }
    if (exact_tstop && (B->tn + B->hprime - tout) * B->hprime > 0.0) {
      B->hprime = (tout - B->tn) * (1.0 - 4.0 * DBL_EPSILON);
    }
    set_ewt(B, B->zn[0]);
    int r = step(B);
    if (r) { memcpy(m_out, B->zn[0], sizeof(double) * B->n); *t_reached = B->tn; return r; }
    ++taken;
    troundoff = 100.0 * DBL_EPSILON * (fabs(B->tn) + fabs(B->h));
  }
}

void om_bdf_stats(const om_bdf *B, om_ts_stats *st) {
  st->nst = B->nst; st->nfe = B->nfe; st->nni = B->nni; st->nli = B->nli; st->ncfn = B->ncfn; st->netf = B->netf;
  st->npe = B->npe; st->nps = B->nps; st->njv = B->njv; st->nje = B->nsetups;
  st->hcur = B->h; st->tcur = B->tn; st->qcur = B->q;
}

/* Fixed-step classical RK4 on the LLG RHS. */
int om_rk4(om_state *S, double *m, double dt, int nsteps) {
  int n = 3 * S->M->n_nodes;
  double *k1 = malloc(sizeof(double) * n), *k2 = malloc(sizeof(double) * n), *k3 = malloc(sizeof(double) * n),
         *k4 = malloc(sizeof(double) * n), *y = malloc(sizeof(double) * n);
  int st = 0;
  for (int s = 0; s < nsteps && !st; ++s) {
    st |= om_rhs(S, m, k1);
    for (int i = 0; i < n; ++i) y[i] = m[i] + 0.5 * dt * k1[i];
    st |= om_rhs(S, y, k2);
    for (int i = 0; i < n; ++i) y[i] = m[i] + 0.5 * dt * k2[i];
    st |= om_rhs(S, y, k3);
    for (int i = 0; i < n; ++i) y[i] = m[i] + dt * k3[i];
    st |= om_rhs(S, y, k4);
    for (int i = 0; i < n; ++i) m[i] += dt / 6.0 * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
  }
  free(k1); free(k2); free(k3); free(k4); free(y);
  return st;
}
