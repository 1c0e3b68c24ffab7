// batch.cu -- batching form: many independent particles of uneven size (each
// its own mesh, material and applied-field direction) advanced in one
// persistent launch.
//
// Each particle's operators and Lindholm BEM are built by the single-handle
// builders (mesh_kernels.cu, bem_kernels.cu) and packed into segmented
// arrays (per-particle offsets; the BEM as one FP32 row-major block per
// particle).  One CTA owns one particle at a time: it takes the next particle
// from a queue ordered by decreasing cost (nb^2 + CG work) and runs whole
// integrator steps for it with block-level synchronisation only, so particles
// of 125 and 9,261 nodes share the GPU without grid barriers.  Inside a CTA
// the right-hand side is the single path's pipeline (nmag_lam.py:734-832):
// rho = -Ms D m, Neumann Jacobi-PCG, BEM product (warp per row, x in shared
// memory), Dirichlet Jacobi-PCG, fused H_eff + LLG.  Time integration is the
// embedded Bogacki-Shampine 3(2) pair with per-particle step control (FSAL),
// and the hysteresis stage logic of hysteresis.py:244-557 runs on the device:
// once max |dm/dt| < stop twice in a row the particle moves to the next field
// of its sweep, H_k = h_max (1 - 2k/(n-1)) along its direction.  The host
// replays a CUDA graph of launches; an autotuner picks the CTA size and the
// per-launch work budget by timing candidates on the batch itself.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "nmg_internal.h"

struct nmg_batch;

namespace nmg {
namespace {

struct PDesc {
  int N, nnz, nb, ld;
  long long on, onz, onb, obem;   // offsets: nodes, nonzeros, boundary nodes, BEM entries
  double Ms, c_exch, C1, C2, C3, anis, ax, ay, az;
  double hdir[3];
  double cost;
  int steps_cap;                  // steps per launch from the work budget
  int pad;
};

struct PState {
  double t, dt, hmag, maxdmdt;
  int stage, done, conv, have_k1;
  long long steps, rejects, rhs, cg_iters;
  long long krylov_iters;   // ROS2 linear-solve iterations
};

struct BatchArgs {
  int P, n_stages, cg_maxits, adaptive;
  int integrator, krylov_maxits;   // 0: Bogacki-Shampine 3(2); 1: ROS2 (linearly implicit)
  double hmax, rtol, atol, cg_rtol, stop_dmdt, dt_max;
  const int *order;
  int *queue;                      // next queue position (reset before each launch)
  const PDesc *desc;
  PState *st;
  const int32_t *row_ptr, *col_idx, *diag, *b_of_node, *node_of_b;
  const double *K, *Gx, *Gy, *Gz, *Dx, *Dy, *Dz, *vol;
  const float *bem;
  double *m, *k0, *k1, *k2, *k3, *y, *phi1, *phi2, *rho, *rhs2, *cr, *cz, *cp, *cq, *b2, *hout;
  // ROS2: field at the step's start, 3x3 block inverses of W, Krylov vectors (3N per particle)
  double *hn, *pinv, *kr, *krh, *kp, *kv, *ks, *kt, *kph, *ksh;
  int *err;
};

constexpr int kMaxWarps = 32;

__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wmax(double v) {
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block sums of two values, result in every thread (fixed order).
__device__ __forceinline__ void bsum2(double &a, double &b, double *sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  a = wsum(a);
  b = wsum(b);
  if (lane == 0) { sm[w] = a; sm[kMaxWarps + w] = b; }
  __syncthreads();
  double ta = 0.0, tb = 0.0;
  for (int q = 0; q < nw; ++q) { ta += sm[q]; tb += sm[kMaxWarps + q]; }
  __syncthreads();
  a = ta;
  b = tb;
}

__device__ __forceinline__ double bmax(double a, double *sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  a = wmax(a);
  if (lane == 0) sm[w] = a;
  __syncthreads();
  double t = 0.0;
  for (int q = 0; q < nw; ++q) t = fmax(t, sm[q]);
  __syncthreads();
  return t;
}

struct PView {   // one particle's slices
  int N, nb, ld;
  const int32_t *rp, *ci, *diag, *bon, *nob;
  const double *K, *Gx, *Gy, *Gz, *Dx, *Dy, *Dz, *vol;
  const float *bem;
  double *phi1, *phi2, *rho, *rhs2, *cr, *cz, *cp, *cq, *b2;
};

__device__ PView view(const BatchArgs &a, int p, const PDesc &d) {
  PView v;
  v.N = d.N; v.nb = d.nb; v.ld = d.ld;
  v.rp = a.row_ptr + d.on + p;
  v.ci = a.col_idx + d.onz;
  v.diag = a.diag + d.on;
  v.bon = a.b_of_node + d.on;
  v.nob = a.node_of_b + d.onb;
  v.K = a.K + d.onz; v.Gx = a.Gx + d.onz; v.Gy = a.Gy + d.onz; v.Gz = a.Gz + d.onz;
  v.Dx = a.Dx + d.onz; v.Dy = a.Dy + d.onz; v.Dz = a.Dz + d.onz;
  v.vol = a.vol + d.on;
  v.bem = a.bem + d.obem;
  v.phi1 = a.phi1 + d.on; v.phi2 = a.phi2 + d.on; v.rho = a.rho + d.on; v.rhs2 = a.rhs2 + d.on;
  v.cr = a.cr + d.on; v.cz = a.cz + d.on; v.cp = a.cp + d.on; v.cq = a.cq + d.on;
  v.b2 = a.b2 + d.onb;
  return v;
}

// (A v)_i: mode 0 the Laplacian K; mode 1 K_II with identity boundary rows.
__device__ __forceinline__ double apply_row(const PView &v, int mode, int i, const double *x) {
  if (mode == 1 && v.bon[i] >= 0) return x[i];
  double s = 0.0;
  for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
    const int j = v.ci[k];
    if (mode == 1 && v.bon[j] >= 0) continue;
    s += v.K[k] * x[j];
  }
  return s;
}

// Jacobi-PCG on one particle by one block; x holds the warm start.  Mode 0:
// b and the solution are centred (constant null space); mode 1: boundary rows
// are identity rows and x is set to b there first.  Returns iterations.
__device__ int block_cg(const PView &v, int mode, const double *b, double *x, double rtol, int maxits,
                        double *sm, bool *failed) {
  const int N = v.N, tid = threadIdx.x, nt = blockDim.x;
  double mean = 0.0;
  if (mode == 0) {
    double s = 0.0, dummy = 0.0;
    for (int i = tid; i < N; i += nt) s += b[i];
    bsum2(s, dummy, sm);
    mean = s / N;
  } else {
    for (int i = tid; i < N; i += nt)
      if (v.bon[i] >= 0) x[i] = b[i];
    __syncthreads();
  }
  double bb = 0.0, rz = 0.0;
  for (int i = tid; i < N; i += nt) {
    const double bi = b[i] - mean;
    const double ri = bi - apply_row(v, mode, i, x);
    const double di = (mode == 1 && v.bon[i] >= 0) ? 1.0 : 1.0 / v.K[v.diag[i]];
    v.cr[i] = ri;
    v.cz[i] = di * ri;
    v.cp[i] = di * ri;
    bb += bi * bi;
    rz += ri * di * ri;
  }
  bsum2(bb, rz, sm);
  const double tol = fmax(rtol * sqrt(bb), 1e-300);
  double rr = 0.0, d2 = 0.0;
  for (int i = tid; i < N; i += nt) rr += v.cr[i] * v.cr[i];
  bsum2(rr, d2, sm);
  int it = 0;
  while (sqrt(rr) > tol) {
    if (it >= maxits || !(rr == rr)) { *failed = true; break; }
    double pq = 0.0, d3 = 0.0;
    for (int i = tid; i < N; i += nt) {
      const double qi = apply_row(v, mode, i, v.cp);
      v.cq[i] = qi;
      pq += v.cp[i] * qi;
    }
    bsum2(pq, d3, sm);
    const double alpha = rz / pq;
    double rzn = 0.0, rrn = 0.0;
    for (int i = tid; i < N; i += nt) {
      x[i] += alpha * v.cp[i];
      const double ri = v.cr[i] - alpha * v.cq[i];
      const double di = (mode == 1 && v.bon[i] >= 0) ? 1.0 : 1.0 / v.K[v.diag[i]];
      v.cr[i] = ri;
      v.cz[i] = di * ri;
      rzn += ri * di * ri;
      rrn += ri * ri;
    }
    bsum2(rzn, rrn, sm);
    const double beta = rzn / rz;
    rz = rzn;
    rr = rrn;
    for (int i = tid; i < N; i += nt) v.cp[i] = v.cz[i] + beta * v.cp[i];
    __syncthreads();
    ++it;
  }
  if (mode == 0) {
    double s = 0.0, dummy = 0.0;
    for (int i = tid; i < N; i += nt) s += x[i];
    bsum2(s, dummy, sm);
    for (int i = tid; i < N; i += nt) x[i] -= s / N;
  }
  __syncthreads();
  return it;
}

// dm/dt = f(y) for one particle (block); H_total to hout when given.
__device__ void prhs(const BatchArgs &a, int p, const PDesc &d, const PView &v, double hmag, const double *y,
                     double *out, double *hout, double *sm, float *xs, PState &st, bool *failed) {
  const int N = v.N, tid = threadIdx.x, nt = blockDim.x;
  // rho = -Ms D y
  for (int i = tid; i < N; i += nt) {
    double s = 0.0;
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const double *yj = y + 3 * (size_t)v.ci[k];
      s += (v.Dx[k] * yj[0] + v.Dy[k] * yj[1]) + v.Dz[k] * yj[2];
    }
    v.rho[i] = -(d.Ms * s);
  }
  __syncthreads();
  st.cg_iters += block_cg(v, 0, v.rho, v.phi1, a.cg_rtol, a.cg_maxits, sm, failed);
  // BEM product phi2b = B phi1b (FP32 matrix and x, FP64 row sums)
  for (int j = tid; j < v.ld; j += nt) xs[j] = j < v.nb ? (float)v.phi1[v.nob[j]] : 0.0f;
  __syncthreads();
  {
    const int lane = tid & 31, w = tid >> 5, nw = nt >> 5;
    for (int r = w; r < v.nb; r += nw) {
      const float4 *row = reinterpret_cast<const float4 *>(v.bem + (size_t)r * v.ld);
      const float4 *x4 = reinterpret_cast<const float4 *>(xs);
      float s0 = 0.f, s1 = 0.f;
      for (int q = lane; q < v.ld / 4; q += 32) {
        const float4 bq = __ldcs(row + q), xq = x4[q];
        s0 = fmaf(bq.x, xq.x, s0); s1 = fmaf(bq.y, xq.y, s1);
        s0 = fmaf(bq.z, xq.z, s0); s1 = fmaf(bq.w, xq.w, s1);
      }
      const double s = wsum((double)s0 + (double)s1);
      if (lane == 0) v.b2[r] = s;
    }
  }
  __syncthreads();
  // Dirichlet right-hand side (op_load_DBC): interior -K_IB phi2b, boundary phi2b
  for (int i = tid; i < N; i += nt) {
    const int bi = v.bon[i];
    if (bi >= 0) { v.rhs2[i] = v.b2[bi]; continue; }
    double s = 0.0;
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const int bj = v.bon[v.ci[k]];
      if (bj >= 0) s += v.K[k] * v.b2[bj];
    }
    v.rhs2[i] = -s;
  }
  __syncthreads();
  st.cg_iters += block_cg(v, 1, v.rhs2, v.phi2, a.cg_rtol, a.cg_maxits, sm, failed);
  // fused H_eff + LLG
  for (int i = tid; i < N; i += nt) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
      const int j = v.ci[k];
      const double kv = v.K[k];
      const double *yj = y + 3 * (size_t)j;
      s0 += kv * yj[0]; s1 += kv * yj[1]; s2 += kv * yj[2];
      const double pj = v.phi1[j] + v.phi2[j];
      g0 += v.Gx[k] * pj; g1 += v.Gy[k] * pj; g2 += v.Gz[k] * pj;
    }
    const double V = v.vol[i];
    const double *m = y + 3 * (size_t)i;
    const double am = (d.ax * m[0] + d.ay * m[1]) + d.az * m[2];
    const double ax[3] = {d.ax, d.ay, d.az};
    double H[3];
    for (int c = 0; c < 3; ++c) {
      const double sc = c == 0 ? s0 : (c == 1 ? s1 : s2), gc = c == 0 ? g0 : (c == 1 ? g1 : g2);
      H[c] = ((hmag * d.hdir[c] - d.c_exch * sc / V) + d.anis * am * (ax[c] - am * m[c])) - gc / V;
    }
    const double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
    const double mxmxH[3] = {m[1] * mxH[2] - m[2] * mxH[1], m[2] * mxH[0] - m[0] * mxH[2],
                             m[0] * mxH[1] - m[1] * mxH[0]};
    const double c3 = d.C3 * (1.0 - ((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]));
    for (int c = 0; c < 3; ++c) {
      out[3 * (size_t)i + c] = (d.C1 * mxH[c] + d.C2 * mxmxH[c]) + c3 * m[c];
      if (hout) hout[3 * (size_t)i + c] = H[c];
    }
  }
  __syncthreads();
  st.rhs++;
}

__device__ __forceinline__ double stage_field(const BatchArgs &a, int stage) {
  return a.n_stages > 1 ? a.hmax * (1.0 - 2.0 * stage / (a.n_stages - 1)) : a.hmax;
}

// Up to d.steps_cap Bogacki-Shampine steps (with the hysteresis stage logic)
// for particle p.
__device__ void particle_run(const BatchArgs &a, int p, double *sm, float *xs, PState &st) {
  const PDesc d = a.desc[p];
  const PView v = view(a, p, d);
  const int n3 = 3 * d.N, tid = threadIdx.x, nt = blockDim.x;
  const size_t o3 = 3 * (size_t)d.on;
  double *m = a.m + o3, *k0 = a.k0 + o3, *k1 = a.k1 + o3, *k2 = a.k2 + o3, *k3 = a.k3 + o3, *y = a.y + o3;
  bool failed = false;
  for (int s = 0; s < d.steps_cap && !st.done; ++s) {
    if (!st.have_k1) {
      prhs(a, p, d, v, st.hmag, m, k0, nullptr, sm, xs, st, &failed);
      st.have_k1 = 1;
    }
    const double dt = st.dt;
    for (int i = tid; i < n3; i += nt) y[i] = m[i] + 0.5 * dt * k0[i];
    __syncthreads();
    prhs(a, p, d, v, st.hmag, y, k1, nullptr, sm, xs, st, &failed);
    for (int i = tid; i < n3; i += nt) y[i] = m[i] + 0.75 * dt * k1[i];
    __syncthreads();
    prhs(a, p, d, v, st.hmag, y, k2, nullptr, sm, xs, st, &failed);
    for (int i = tid; i < n3; i += nt)
      y[i] = m[i] + dt * (((2.0 / 9.0) * k0[i] + (1.0 / 3.0) * k1[i]) + (4.0 / 9.0) * k2[i]);
    __syncthreads();
    prhs(a, p, d, v, st.hmag, y, k3, nullptr, sm, xs, st, &failed);
    double en = 0.0;
    if (a.adaptive) {
      for (int i = tid; i < n3; i += nt) {
        const double e = dt * ((((2.0 / 9.0 - 7.0 / 24.0) * k0[i] + (1.0 / 3.0 - 0.25) * k1[i]) +
                               (4.0 / 9.0 - 1.0 / 3.0) * k2[i]) - 0.125 * k3[i]);
        en = fmax(en, fabs(e) / (a.atol + a.rtol * fmax(fabs(m[i]), fabs(y[i]))));
      }
      en = bmax(en, sm);
    }
    if (failed || !(en == en)) {
      if (tid == 0) atomicOr(a.err, ERR_NONFINITE);
      st.done = 1;
      break;
    }
    if (en <= 1.0) {   // accept: m <- y, FSAL
      double mx = 0.0;
      for (int i = tid; i < d.N; i += nt) {
        for (int c = 0; c < 3; ++c) {
          m[3 * (size_t)i + c] = y[3 * (size_t)i + c];
          k0[3 * (size_t)i + c] = k3[3 * (size_t)i + c];
        }
        const double *f = k3 + 3 * (size_t)i;
        mx = fmax(mx, sqrt((f[0] * f[0] + f[1] * f[1]) + f[2] * f[2]));
      }
      mx = bmax(mx, sm);
      st.t += dt;
      st.steps++;
      st.maxdmdt = mx;
      st.conv = mx < a.stop_dmdt ? st.conv + 1 : 0;
      if (st.conv >= 2) {   // converged twice in a row: next field of the sweep
        st.conv = 0;
        st.stage++;
        if (st.stage >= a.n_stages) st.done = 1;
        else { st.hmag = stage_field(a, st.stage); st.have_k1 = 0; }
      }
    } else {
      st.rejects++;
    }
    if (a.adaptive) {
      const double fac = en > 0.0 ? 0.9 * pow(en, -1.0 / 3.0) : 5.0;
      st.dt = fmin(a.dt_max, dt * fmin(5.0, fmax(0.2, fac)));
    }
    __syncthreads();
  }
}

// ---- linearly implicit integrator: ROS2 ----
// The two-stage Rosenbrock W-method of Verwer, Spee, Blom and Hundsdorfer
// (1999): gamma = 1 + 1/sqrt(2), W = I - gamma tau J,
//   W k1 = f(y_n),  W k2 = f(y_n + tau k1) - 2 k1,
//   y_{n+1} = y_n + tau (3/2 k1 + 1/2 k2),  error estimate tau/2 (k1 + k2).
// It is L-stable and second order for any matrix J, so J is the exchange and
// site linearisation of f at (y_n, H_n) with the demagnetising and
// anisotropy fields frozen -- the Jacobian of the single-film path
// (nsim.ml:967-1050) -- and the step is limited by accuracy, not by the
// exchange stiffness that bounds the explicit integrator.  W k = b is solved
// by block-level BiCGSTAB preconditioned with the 3x3 node blocks of W.
constexpr double kRos2Gamma = 1.7071067811865475;   // 1 + 1/sqrt(2)

__device__ __forceinline__ void bcross(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
// dF = C1 (w x H + m x hv) + C2 (w x (m x H) + m x (w x H + m x hv))
__device__ __forceinline__ void bjac(const double *m, const double *H, const double *w, const double *hv, double C1,
                                     double C2, double *out) {
  double wxH[3], mxhv[3], mxH[3], t1[3], u[3], t2[3];
  bcross(w, H, wxH);
  bcross(m, hv, mxhv);
  bcross(m, H, mxH);
  bcross(w, mxH, t1);
  for (int c = 0; c < 3; ++c) u[c] = wxH[c] + mxhv[c];
  bcross(m, u, t2);
  for (int c = 0; c < 3; ++c) out[c] = C1 * (wxH[c] + mxhv[c]) + C2 * (t1[c] + t2[c]);
}
// (W x)_i = x_i - gt (J x)_i
__device__ __forceinline__ void wapply(const PView &v, const PDesc &d, int i, const double *m, const double *H,
                                       double gt, const double *x, double *out) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int k = v.rp[i]; k < v.rp[i + 1]; ++k) {
    const double *xj = x + 3 * (size_t)v.ci[k];
    const double kv = v.K[k];
    s0 += kv * xj[0]; s1 += kv * xj[1]; s2 += kv * xj[2];
  }
  const double V = v.vol[i];
  const double hv[3] = {-d.c_exch * s0 / V, -d.c_exch * s1 / V, -d.c_exch * s2 / V};
  double jx[3];
  bjac(m + 3 * (size_t)i, H + 3 * (size_t)i, x + 3 * (size_t)i, hv, d.C1, d.C2, jx);
  for (int c = 0; c < 3; ++c) out[c] = x[3 * (size_t)i + c] - gt * jx[c];
}
// Pinv_i = inverse of node i's 3x3 block of W (row-major, 9 values)
__device__ void pblock(const PView &v, const PDesc &d, int i, const double *m, const double *H, double gt,
                       double *Pi) {
  const double kap = -d.c_exch * v.K[v.diag[i]] / v.vol[i];
  double P[3][3];
  for (int c = 0; c < 3; ++c) {
    double e[3] = {0.0, 0.0, 0.0};
    e[c] = 1.0;
    const double he[3] = {kap * e[0], kap * e[1], kap * e[2]};
    double je[3];
    bjac(m + 3 * (size_t)i, H + 3 * (size_t)i, e, he, d.C1, d.C2, je);
    for (int r = 0; r < 3; ++r) P[r][c] = (r == c ? 1.0 : 0.0) - gt * je[r];
  }
  const double c00 = P[1][1] * P[2][2] - P[1][2] * P[2][1];
  const double c01 = P[1][2] * P[2][0] - P[1][0] * P[2][2];
  const double c02 = P[1][0] * P[2][1] - P[1][1] * P[2][0];
  const double inv = 1.0 / (P[0][0] * c00 + P[0][1] * c01 + P[0][2] * c02);
  Pi[0] = c00 * inv; Pi[1] = (P[0][2] * P[2][1] - P[0][1] * P[2][2]) * inv; Pi[2] = (P[0][1] * P[1][2] - P[0][2] * P[1][1]) * inv;
  Pi[3] = c01 * inv; Pi[4] = (P[0][0] * P[2][2] - P[0][2] * P[2][0]) * inv; Pi[5] = (P[0][2] * P[1][0] - P[0][0] * P[1][2]) * inv;
  Pi[6] = c02 * inv; Pi[7] = (P[0][1] * P[2][0] - P[0][0] * P[2][1]) * inv; Pi[8] = (P[0][0] * P[1][1] - P[0][1] * P[1][0]) * inv;
}
__device__ __forceinline__ void pmul(const double *Pinv, int i, const double *x, double *out) {
  const double *Pi = Pinv + 9 * (size_t)i, *xi = x + 3 * (size_t)i;
  for (int r = 0; r < 3; ++r) out[3 * (size_t)i + r] = (Pi[3 * r] * xi[0] + Pi[3 * r + 1] * xi[1]) + Pi[3 * r + 2] * xi[2];
}

struct KrylovVecs { double *r, *rh, *p, *v, *s, *t, *ph, *sh; };

// W x = b by right-preconditioned BiCGSTAB on one particle (block); x holds
// the initial guess.  Stops at |r| <= rtol |b|; returns iterations, sets
// *failed on breakdown or when maxits is reached.
__device__ int block_bicgstab(const PView &v, const PDesc &d, const double *m, const double *H, double gt,
                              const double *Pinv, const double *b, double *x, double rtol, int maxits,
                              const KrylovVecs &K, double *sm, bool *failed) {
  const int N = v.N, tid = threadIdx.x, nt = blockDim.x;
  double bb = 0.0, rr = 0.0;
  for (int i = tid; i < N; i += nt) {
    double wx[3];
    wapply(v, d, i, m, H, gt, x, wx);
    for (int c = 0; c < 3; ++c) {
      const size_t o = 3 * (size_t)i + c;
      const double r = b[o] - wx[c];
      K.r[o] = r; K.rh[o] = r; K.p[o] = 0.0; K.v[o] = 0.0;
      bb += b[o] * b[o];
      rr += r * r;
    }
  }
  bsum2(bb, rr, sm);
  const double tol = rtol * sqrt(bb);
  double rho = 1.0, alpha = 1.0, omega = 1.0;
  int it = 0;
  while (sqrt(rr) > tol) {
    if (it >= maxits || !(rr == rr)) { *failed = true; break; }
    double rho1 = 0.0, dum = 0.0;
    for (int o = tid; o < 3 * N; o += nt) rho1 += K.rh[o] * K.r[o];
    bsum2(rho1, dum, sm);
    if (rho1 == 0.0 || omega == 0.0) { *failed = true; break; }
    const double beta = (rho1 / rho) * (alpha / omega);
    for (int o = tid; o < 3 * N; o += nt) K.p[o] = K.r[o] + beta * (K.p[o] - omega * K.v[o]);
    __syncthreads();
    for (int i = tid; i < N; i += nt) pmul(Pinv, i, K.p, K.ph);
    __syncthreads();
    double rv = 0.0;
    for (int i = tid; i < N; i += nt) {
      double w[3];
      wapply(v, d, i, m, H, gt, K.ph, w);
      for (int c = 0; c < 3; ++c) {
        const size_t o = 3 * (size_t)i + c;
        K.v[o] = w[c];
        rv += K.rh[o] * w[c];
      }
    }
    bsum2(rv, dum, sm);
    if (rv == 0.0) { *failed = true; break; }
    alpha = rho1 / rv;
    double ss = 0.0;
    for (int o = tid; o < 3 * N; o += nt) {
      const double sv = K.r[o] - alpha * K.v[o];
      K.s[o] = sv;
      ss += sv * sv;
    }
    bsum2(ss, dum, sm);
    ++it;
    if (sqrt(ss) <= tol) {
      for (int o = tid; o < 3 * N; o += nt) x[o] += alpha * K.ph[o];
      rr = ss;
      __syncthreads();
      break;
    }
    for (int i = tid; i < N; i += nt) pmul(Pinv, i, K.s, K.sh);
    __syncthreads();
    double ts = 0.0, tt = 0.0;
    for (int i = tid; i < N; i += nt) {
      double w[3];
      wapply(v, d, i, m, H, gt, K.sh, w);
      for (int c = 0; c < 3; ++c) {
        const size_t o = 3 * (size_t)i + c;
        K.t[o] = w[c];
        ts += w[c] * K.s[o];
        tt += w[c] * w[c];
      }
    }
    bsum2(ts, tt, sm);
    omega = tt > 0.0 ? ts / tt : 0.0;
    double rn = 0.0;
    for (int o = tid; o < 3 * N; o += nt) {
      x[o] += alpha * K.ph[o] + omega * K.sh[o];
      const double r = K.s[o] - omega * K.t[o];
      K.r[o] = r;
      rn += r * r;
    }
    bsum2(rn, dum, sm);
    rr = rn;
    rho = rho1;
  }
  __syncthreads();
  return it;
}

// Up to d.steps_cap ROS2 steps (with the hysteresis stage logic) for particle p.
__device__ void particle_run_ros2(const BatchArgs &a, int p, double *sm, float *xs, PState &st) {
  const PDesc d = a.desc[p];
  const PView v = view(a, p, d);
  const int n3 = 3 * d.N, N = d.N, tid = threadIdx.x, nt = blockDim.x;
  const size_t o3 = 3 * (size_t)d.on;
  double *m = a.m + o3, *f0 = a.k0 + o3, *k1 = a.k1 + o3, *k2 = a.k2 + o3, *f1 = a.k3 + o3, *y = a.y + o3;
  double *H = a.hn + o3, *Pinv = a.pinv + 3 * o3;
  const KrylovVecs K = {a.kr + o3, a.krh + o3, a.kp + o3, a.kv + o3, a.ks + o3, a.kt + o3, a.kph + o3, a.ksh + o3};
  const double krtol = 1e-3 * fmin(a.rtol, a.atol) > 1e-12 ? 1e-3 * fmin(a.rtol, a.atol) : 1e-12;
  bool failed = false;
  for (int s = 0; s < d.steps_cap && !st.done; ++s) {
    if (!st.have_k1) {   // f and H at the step's start (after a new field of the sweep)
      prhs(a, p, d, v, st.hmag, m, f0, H, sm, xs, st, &failed);
      st.have_k1 = 1;
    }
    const double tau = st.dt, gt = kRos2Gamma * tau;
    for (int i = tid; i < N; i += nt) pblock(v, d, i, m, H, gt, Pinv + 9 * (size_t)i);
    for (int o = tid; o < n3; o += nt) k1[o] = f0[o];
    __syncthreads();
    st.krylov_iters += block_bicgstab(v, d, m, H, gt, Pinv, f0, k1, krtol, a.krylov_maxits, K, sm, &failed);
    for (int o = tid; o < n3; o += nt) y[o] = m[o] + tau * k1[o];
    __syncthreads();
    prhs(a, p, d, v, st.hmag, y, f1, nullptr, sm, xs, st, &failed);
    for (int o = tid; o < n3; o += nt) {
      f1[o] -= 2.0 * k1[o];
      k2[o] = f1[o];
    }
    __syncthreads();
    st.krylov_iters += block_bicgstab(v, d, m, H, gt, Pinv, f1, k2, krtol, a.krylov_maxits, K, sm, &failed);
    double en = 0.0;
    for (int o = tid; o < n3; o += nt) {
      const double yn = m[o] + tau * (1.5 * k1[o] + 0.5 * k2[o]);
      y[o] = yn;
      if (a.adaptive) en = fmax(en, fabs(0.5 * tau * (k1[o] + k2[o])) / (a.atol + a.rtol * fmax(fabs(m[o]), fabs(yn))));
    }
    if (a.adaptive) en = bmax(en, sm);
    else __syncthreads();
    if (failed || !(en == en)) {
      if (tid == 0) atomicOr(a.err, failed ? ERR_CG_MAXITS : ERR_NONFINITE);
      st.done = 1;
      break;
    }
    if (en <= 1.0) {   // accept: m <- y, then f and H there (the next step's start)
      for (int o = tid; o < n3; o += nt) m[o] = y[o];
      __syncthreads();
      prhs(a, p, d, v, st.hmag, m, f0, H, sm, xs, st, &failed);
      double mx = 0.0;
      for (int i = tid; i < N; i += nt) {
        const double *f = f0 + 3 * (size_t)i;
        mx = fmax(mx, sqrt((f[0] * f[0] + f[1] * f[1]) + f[2] * f[2]));
      }
      mx = bmax(mx, sm);
      st.t += tau;
      st.steps++;
      st.maxdmdt = mx;
      st.conv = mx < a.stop_dmdt ? st.conv + 1 : 0;
      if (st.conv >= 2) {
        st.conv = 0;
        st.stage++;
        if (st.stage >= a.n_stages) st.done = 1;
        else { st.hmag = stage_field(a, st.stage); st.have_k1 = 0; }
      }
    } else {
      st.rejects++;
    }
    if (a.adaptive) {   // first-order error estimate
      const double fac = en > 0.0 ? 0.9 * sqrt(1.0 / en) : 5.0;
      st.dt = fmin(a.dt_max, tau * fmin(5.0, fmax(0.2, fac)));
    }
    __syncthreads();
  }
}

__global__ void k_batch_run(BatchArgs a) {
  extern __shared__ float xs[];
  __shared__ double sm[2 * kMaxWarps];
  __shared__ int sp;
  __shared__ PState st;
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = atomicAdd(a.queue, 1);
      sp = q < a.P ? a.order[q] : -1;
      if (sp >= 0) st = a.st[sp];
    }
    __syncthreads();
    const int p = sp;
    if (p < 0) break;
    // every thread works on a private copy of the scalars; thread 0's is stored
    PState mine = st;
    if (!mine.done) {
      if (a.integrator == 1) particle_run_ros2(a, p, sm, xs, mine);
      else particle_run(a, p, sm, xs, mine);
    }
    __syncthreads();
    if (threadIdx.x == 0) a.st[p] = mine;
    __syncthreads();
  }
}

// One RHS evaluation per particle at its current m and stage field.
__global__ void k_batch_eval(BatchArgs a, double *dmdt) {
  extern __shared__ float xs[];
  __shared__ double sm[2 * kMaxWarps];
  __shared__ int sp;
  for (;;) {
    if (threadIdx.x == 0) {
      const int q = atomicAdd(a.queue, 1);
      sp = q < a.P ? a.order[q] : -1;
    }
    __syncthreads();
    const int p = sp;
    if (p < 0) break;
    const PDesc d = a.desc[p];
    const PView v = view(a, p, d);
    PState st = a.st[p];
    bool failed = false;
    prhs(a, p, d, v, st.hmag, a.m + 3 * (size_t)d.on, dmdt + 3 * (size_t)d.on, a.hout + 3 * (size_t)d.on, sm, xs,
         st, &failed);
    if (failed && threadIdx.x == 0) atomicOr(a.err, ERR_CG_MAXITS);
    __syncthreads();
  }
}

}  // namespace
}  // namespace nmg

struct nmg_batch {
  int P = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::string last_error;
  nmg_batch_options opt{};
  std::vector<nmg::PDesc> hdesc;
  int ld_max = 8;
  long long Ntot = 0;
  nmg::DevBuf<int32_t> row_ptr, col_idx, diag, b_of_node, node_of_b, order, queue;
  nmg::DevBuf<double> K, Gx, Gy, Gz, Dx, Dy, Dz, vol;
  nmg::DevBuf<float> bem;
  nmg::DevBuf<double> m, k0, k1, k2, k3, y, phi1, phi2, rho, rhs2, cr, cz, cp, cq, b2, hout, dmdt;
  nmg::DevBuf<double> hn, pinv, kr, krh, kp, kv, ks, kt, kph, ksh;   // ROS2 integrator only
  nmg::DevBuf<nmg::PDesc> desc;
  nmg::DevBuf<nmg::PState> st;
  nmg::DevBuf<int> err;
  int threads = 256;
  double budget = 0.0;
  int blocks = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_launches = 0, graph_threads = 0;
  nmg::BatchArgs args() const;
};

namespace {

thread_local std::string g_batch_error;

int bfail(nmg_batch *b, int code, const std::string &msg) {
  if (b) b->last_error = msg;
  else g_batch_error = msg;
  return code;
}

}  // namespace

nmg::BatchArgs nmg_batch::args() const {
  nmg::BatchArgs a{};
  a.P = P; a.n_stages = opt.n_stages; a.cg_maxits = opt.cg_maxits; a.adaptive = opt.fixed_dt > 0.0 ? 0 : 1;
  a.integrator = opt.integrator;
  a.krylov_maxits = opt.krylov_maxits > 0 ? opt.krylov_maxits : 200;
  a.hn = hn; a.pinv = pinv; a.kr = kr; a.krh = krh; a.kp = kp; a.kv = kv; a.ks = ks; a.kt = kt; a.kph = kph;
  a.ksh = ksh;
  a.hmax = opt.h_max; a.rtol = opt.rtol; a.atol = opt.atol; a.cg_rtol = opt.cg_rtol;
  a.stop_dmdt = opt.stop_dmdt; a.dt_max = opt.dt_max;
  a.order = order; a.queue = queue; a.desc = desc; a.st = st;
  a.row_ptr = row_ptr; a.col_idx = col_idx; a.diag = diag; a.b_of_node = b_of_node; a.node_of_b = node_of_b;
  a.K = K; a.Gx = Gx; a.Gy = Gy; a.Gz = Gz; a.Dx = Dx; a.Dy = Dy; a.Dz = Dz; a.vol = vol; a.bem = bem;
  a.m = m; a.k0 = k0; a.k1 = k1; a.k2 = k2; a.k3 = k3; a.y = y; a.phi1 = phi1; a.phi2 = phi2; a.rho = rho;
  a.rhs2 = rhs2; a.cr = cr; a.cz = cz; a.cp = cp; a.cq = cq; a.b2 = b2; a.hout = hout; a.err = err;
  return a;
}

namespace {

// Steps per launch for each particle from the work budget (cost units).
void apply_budget(nmg_batch *b) {
  for (auto &d : b->hdesc) {
    const double s = b->budget > 0.0 ? b->budget / d.cost : 1.0;
    d.steps_cap = (int)std::max(1.0, std::min(1e6, std::floor(s)));
  }
  cudaMemcpyAsync(b->desc.p, b->hdesc.data(), sizeof(nmg::PDesc) * b->P, cudaMemcpyHostToDevice, b->stream);
}

size_t smem_bytes(const nmg_batch *b) { return sizeof(float) * (size_t)b->ld_max; }

int launch_run(nmg_batch *b) {
  nmg::BatchArgs a = b->args();
  cudaMemsetAsync(b->queue.p, 0, sizeof(int), b->stream);
  nmg::k_batch_run<<<b->blocks, b->threads, smem_bytes(b), b->stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

int sync_check(nmg_batch *b, const char *where) {
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bfail(b, 100, std::string(where) + ": " + cudaGetErrorString(e));
  int derr = 0;
  cudaMemcpy(&derr, b->err.p, sizeof(int), cudaMemcpyDeviceToHost);
  if (derr) {
    cudaMemsetAsync(b->err.p, 0, sizeof(int), b->stream);
    cudaStreamSynchronize(b->stream);
    return bfail(b, (derr & nmg::ERR_NONFINITE) ? 6 : 5,
                 std::string(where) + ((derr & nmg::ERR_NONFINITE) ? ": non-finite state or CG failure"
                                                                    : ": CG reached its iteration limit"));
  }
  return 0;
}

void drop_graph(nmg_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_launches = 0;
}

int set_threads(nmg_batch *b, int threads) {
  int per = 0;
  if (cudaFuncSetAttribute(nmg::k_batch_run, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(b)) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, nmg::k_batch_run, threads, smem_bytes(b)) != cudaSuccess ||
      per < 1) {
    cudaGetLastError();
    return bfail(b, 4, "batch kernel cannot run with " + std::to_string(threads) + " threads");
  }
  cudaFuncSetAttribute(nmg::k_batch_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(b));
  b->threads = threads;
  b->blocks = std::min(b->P, per * b->sm_count);
  drop_graph(b);
  return 0;
}

}  // namespace

extern "C" {

const char *nmg_batch_last_error(const nmg_batch *b) { return b ? b->last_error.c_str() : g_batch_error.c_str(); }

int nmg_batch_create(const nmg_particle *parts, int n, const nmg_batch_options *opt, nmg_batch **out) {
  if (!out || !parts || !opt || n < 1) return bfail(nullptr, -1, "nmg_batch_create: bad arguments");
  *out = nullptr;
  if (opt->n_stages < 1 || opt->cg_maxits < 1 || !(opt->cg_rtol > 0.0))
    return bfail(nullptr, -2, "nmg_batch_create: need n_stages >= 1, cg_maxits >= 1, cg_rtol > 0");
  if (opt->integrator < 0 || opt->integrator > 1 || opt->krylov_maxits < 0)
    return bfail(nullptr, -2, "nmg_batch_create: integrator must be 0 (Bogacki-Shampine) or 1 (ROS2)");
  nmg_batch *b = new nmg_batch();
  b->P = n;
  b->opt = *opt;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return bfail(nullptr, 101, "nmg_batch_create: stream creation failed");
  }
  // ---- build every particle on a transient handle; gather sizes ----
  struct Host {
    std::vector<int32_t> rp, ci, dg, bon, nob;
    std::vector<double> K, G, D, vol;
    std::vector<float> bem;
  };
  std::vector<Host> hs(n);
  long long on = 0, onz = 0, onb = 0, obem = 0;
  b->hdesc.resize(n);
  for (int p = 0; p < n; ++p) {
    const nmg_particle &q = parts[p];
    if (!q.coords || !q.tets || q.n_nodes < 4 || q.n_tets < 1) {
      nmg_batch_destroy(b);
      return bfail(nullptr, -2, "nmg_batch_create: particle " + std::to_string(p) + " has no mesh");
    }
    nmg_handle *h = new nmg_handle();
    h->mat = q.mat;
    h->opt.do_demag = 1;
    h->sm_count = b->sm_count;
    h->stream = b->stream;
    h->mesh.N = q.n_nodes;
    h->mesh.T = q.n_tets;
    std::string err;
    int rc = h->ws.err.alloc(1) == cudaSuccess ? 0 : 100;
    if (!rc) cudaMemsetAsync(h->ws.err.p, 0, sizeof(int), b->stream);
    if (!rc) rc = nmg::build_mesh(h, q.coords, q.tets, err);
    if (!rc) {
      h->mesh.ld = (h->mesh.nb + 7) / 8 * 8;
      rc = nmg::fill_bem(h, err);
    }
    if (rc) {
      h->stream = nullptr;
      delete h;
      nmg_batch_destroy(b);
      return bfail(nullptr, rc, "nmg_batch_create: particle " + std::to_string(p) + ": " + err);
    }
    nmg::Mesh &M = h->mesh;
    Host &H = hs[p];
    H.rp.resize(M.N + 1); H.ci.resize(M.nnz); H.dg.resize(M.N); H.bon.resize(M.N); H.nob.resize(M.nb);
    H.K.resize(M.nnz); H.G.resize(3 * (size_t)M.nnz); H.D.resize(3 * (size_t)M.nnz); H.vol.resize(M.N);
    std::vector<double> bem64((size_t)M.nb * M.ld);
    cudaMemcpy(H.rp.data(), M.row_ptr.p, sizeof(int32_t) * (M.N + 1), cudaMemcpyDeviceToHost);
    cudaMemcpy(H.ci.data(), M.col_idx.p, sizeof(int32_t) * M.nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.dg.data(), M.diag_pos.p, sizeof(int32_t) * M.N, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.bon.data(), M.b_of_node.p, sizeof(int32_t) * M.N, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.nob.data(), M.node_of_b.p, sizeof(int32_t) * M.nb, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.K.data(), M.K.p, sizeof(double) * M.nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.G.data(), M.G.p, sizeof(double) * 3 * M.nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.D.data(), M.D.p, sizeof(double) * 3 * M.nnz, cudaMemcpyDeviceToHost);
    cudaMemcpy(H.vol.data(), M.vol.p, sizeof(double) * M.N, cudaMemcpyDeviceToHost);
    cudaMemcpy(bem64.data(), M.bem.p, sizeof(double) * bem64.size(), cudaMemcpyDeviceToHost);
    H.bem.assign(bem64.begin(), bem64.end());
    nmg::PDesc &d = b->hdesc[p];
    d.N = M.N; d.nnz = M.nnz; d.nb = M.nb; d.ld = M.ld;
    d.on = on; d.onz = onz; d.onb = onb; d.obem = obem;
    d.Ms = q.mat.Ms; d.c_exch = q.mat.exch_coeff; d.C1 = q.mat.C1; d.C2 = q.mat.C2; d.C3 = q.mat.C3;
    d.anis = q.mat.K1 != 0.0 ? q.mat.anis_coeff : 0.0;
    d.ax = q.mat.axis[0]; d.ay = q.mat.axis[1]; d.az = q.mat.axis[2];
    const double hn = std::sqrt(q.h_dir[0] * q.h_dir[0] + q.h_dir[1] * q.h_dir[1] + q.h_dir[2] * q.h_dir[2]);
    for (int c = 0; c < 3; ++c) d.hdir[c] = hn > 0.0 ? q.h_dir[c] / hn : 0.0;
    d.cost = (double)M.nb * M.nb + 60.0 * M.nnz;   // BEM entries + ~two CG solves of ~30 iterations
    d.steps_cap = 1;
    b->ld_max = std::max(b->ld_max, M.ld);
    on += M.N; onz += M.nnz; onb += M.nb; obem += (long long)M.nb * M.ld;
    h->stream = nullptr;   // the batch owns the stream
    delete h;
  }
  b->Ntot = on;
  // ---- pack ----
  int rc = 0;
  auto up32 = [&](nmg::DevBuf<int32_t> &dst, size_t cnt, auto getter) {
    std::vector<int32_t> all;
    all.reserve(cnt);
    for (int p = 0; p < n; ++p) getter(p, all);
    if (dst.alloc(std::max<size_t>(all.size(), 1)) ||
        cudaMemcpy(dst.p, all.data(), sizeof(int32_t) * all.size(), cudaMemcpyHostToDevice))
      rc = 100;
  };
  auto up64 = [&](nmg::DevBuf<double> &dst, size_t cnt, auto getter) {
    std::vector<double> all;
    all.reserve(cnt);
    for (int p = 0; p < n; ++p) getter(p, all);
    if (dst.alloc(std::max<size_t>(all.size(), 1)) ||
        cudaMemcpy(dst.p, all.data(), sizeof(double) * all.size(), cudaMemcpyHostToDevice))
      rc = 100;
  };
  up32(b->row_ptr, on + n, [&](int p, std::vector<int32_t> &v) { v.insert(v.end(), hs[p].rp.begin(), hs[p].rp.end()); });
  up32(b->col_idx, onz, [&](int p, std::vector<int32_t> &v) { v.insert(v.end(), hs[p].ci.begin(), hs[p].ci.end()); });
  up32(b->diag, on, [&](int p, std::vector<int32_t> &v) { v.insert(v.end(), hs[p].dg.begin(), hs[p].dg.end()); });
  up32(b->b_of_node, on, [&](int p, std::vector<int32_t> &v) { v.insert(v.end(), hs[p].bon.begin(), hs[p].bon.end()); });
  up32(b->node_of_b, onb, [&](int p, std::vector<int32_t> &v) { v.insert(v.end(), hs[p].nob.begin(), hs[p].nob.end()); });
  up64(b->K, onz, [&](int p, std::vector<double> &v) { v.insert(v.end(), hs[p].K.begin(), hs[p].K.end()); });
  nmg::DevBuf<double> *Gs[3] = {&b->Gx, &b->Gy, &b->Gz}, *Ds[3] = {&b->Dx, &b->Dy, &b->Dz};
  for (int c = 0; c < 3; ++c) {
    up64(*Gs[c], onz, [&](int p, std::vector<double> &v) {
      const size_t z = hs[p].K.size();
      v.insert(v.end(), hs[p].G.begin() + c * z, hs[p].G.begin() + (c + 1) * z);
    });
    up64(*Ds[c], onz, [&](int p, std::vector<double> &v) {
      const size_t z = hs[p].K.size();
      v.insert(v.end(), hs[p].D.begin() + c * z, hs[p].D.begin() + (c + 1) * z);
    });
  }
  up64(b->vol, on, [&](int p, std::vector<double> &v) { v.insert(v.end(), hs[p].vol.begin(), hs[p].vol.end()); });
  {
    std::vector<float> all;
    all.reserve(obem);
    for (int p = 0; p < n; ++p) all.insert(all.end(), hs[p].bem.begin(), hs[p].bem.end());
    if (b->bem.alloc(std::max<size_t>(all.size(), 4)) ||
        cudaMemcpy(b->bem.p, all.data(), sizeof(float) * all.size(), cudaMemcpyHostToDevice))
      rc = 100;
  }
  const size_t n3 = 3 * (size_t)on;
  for (nmg::DevBuf<double> *v : {&b->m, &b->k0, &b->k1, &b->k2, &b->k3, &b->y, &b->hout, &b->dmdt})
    if (v->alloc(n3)) rc = 100;
  if (opt->integrator == 1) {
    for (nmg::DevBuf<double> *v : {&b->hn, &b->kr, &b->krh, &b->kp, &b->kv, &b->ks, &b->kt, &b->kph, &b->ksh})
      if (v->alloc(n3)) rc = 100;
    if (b->pinv.alloc(3 * n3)) rc = 100;
  }
  for (nmg::DevBuf<double> *v : {&b->phi1, &b->phi2, &b->rho, &b->rhs2, &b->cr, &b->cz, &b->cp, &b->cq})
    if (v->alloc(on) || cudaMemset(v->p, 0, sizeof(double) * on)) rc = 100;
  if (b->b2.alloc(std::max<long long>(onb, 1))) rc = 100;
  if (b->err.alloc(1) || cudaMemset(b->err.p, 0, sizeof(int))) rc = 100;
  if (b->queue.alloc(1)) rc = 100;
  // queue order: decreasing cost
  std::vector<int32_t> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return b->hdesc[x].cost > b->hdesc[y].cost; });
  if (b->order.alloc(n) || cudaMemcpy(b->order.p, ord.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice)) rc = 100;
  // per-particle state
  std::vector<nmg::PState> st(n);
  for (int p = 0; p < n; ++p) {
    st[p] = nmg::PState{};
    st[p].dt = opt->fixed_dt > 0.0 ? opt->fixed_dt : opt->dt0;
    st[p].hmag = opt->n_stages > 1 ? opt->h_max : opt->h_max;
  }
  if (b->st.alloc(n) || cudaMemcpy(b->st.p, st.data(), sizeof(nmg::PState) * n, cudaMemcpyHostToDevice)) rc = 100;
  if (b->desc.alloc(n)) rc = 100;
  if (rc) {
    nmg_batch_destroy(b);
    return bfail(nullptr, 100, "nmg_batch_create: device allocation failed");
  }
  b->budget = opt->budget;
  apply_budget(b);
  rc = set_threads(b, opt->threads > 0 ? opt->threads : 256);
  if (rc) {
    std::string e = b->last_error;
    nmg_batch_destroy(b);
    return bfail(nullptr, rc, e);
  }
  // the setup copies above ran on the legacy stream, which the batch's
  // non-blocking stream does not wait for: finish them before any launch
  if (cudaStreamSynchronize(b->stream) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    nmg_batch_destroy(b);
    return bfail(nullptr, 100, "nmg_batch_create: setup failed");
  }
  *out = b;
  return 0;
}

int nmg_batch_destroy(nmg_batch *b) {
  if (!b) return -1;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graph(b);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return 0;
}

int nmg_batch_info(const nmg_batch *b, int64_t *nodes_total, int32_t *nodes, int32_t *nb) {
  if (!b) return -1;
  if (nodes_total) *nodes_total = b->Ntot;
  for (int p = 0; p < b->P; ++p) {
    if (nodes) nodes[p] = b->hdesc[p].N;
    if (nb) nb[p] = b->hdesc[p].nb;
  }
  return 0;
}

int nmg_batch_set_m(nmg_batch *b, const double *m) {
  if (!b || !m) return -1;
  for (long long k = 0; k < 3 * b->Ntot; ++k)
    if (!(m[k] == m[k])) return bfail(b, -4, "nmg_batch_set_m: non-finite magnetisation");
  cudaMemcpyAsync(b->m.p, m, sizeof(double) * 3 * b->Ntot, cudaMemcpyHostToDevice, b->stream);
  // the FSAL slope belongs to the old state
  std::vector<nmg::PState> st(b->P);
  cudaMemcpyAsync(st.data(), b->st.p, sizeof(nmg::PState) * b->P, cudaMemcpyDeviceToHost, b->stream);
  cudaStreamSynchronize(b->stream);
  for (auto &s : st) s.have_k1 = 0;
  cudaMemcpyAsync(b->st.p, st.data(), sizeof(nmg::PState) * b->P, cudaMemcpyHostToDevice, b->stream);
  return sync_check(b, "nmg_batch_set_m");
}

int nmg_batch_get_m(const nmg_batch *b, double *m) {
  if (!b || !m) return -1;
  nmg_batch *bb = const_cast<nmg_batch *>(b);
  cudaMemcpyAsync(m, b->m.p, sizeof(double) * 3 * b->Ntot, cudaMemcpyDeviceToHost, b->stream);
  return sync_check(bb, "nmg_batch_get_m");
}

int nmg_batch_eval(nmg_batch *b, double *dmdt, double *h_total) {
  if (!b) return -1;
  nmg::BatchArgs a = b->args();
  cudaMemsetAsync(b->queue.p, 0, sizeof(int), b->stream);
  nmg::k_batch_eval<<<b->blocks, b->threads, smem_bytes(b), b->stream>>>(a, b->dmdt);
  if (cudaGetLastError() != cudaSuccess) return bfail(b, 100, "nmg_batch_eval: launch failed");
  int rc = sync_check(b, "nmg_batch_eval");
  if (rc) return rc;
  if (dmdt) cudaMemcpy(dmdt, b->dmdt.p, sizeof(double) * 3 * b->Ntot, cudaMemcpyDeviceToHost);
  if (h_total) cudaMemcpy(h_total, b->hout.p, sizeof(double) * 3 * b->Ntot, cudaMemcpyDeviceToHost);
  return 0;
}

int nmg_batch_run(nmg_batch *b, int launches) {
  if (!b || launches < 0) return -1;
  if (launches == 0) return 0;
  // a CUDA graph of `launches` queue resets + persistent launches, rebuilt
  // when the launch count or the CTA size changes
  if (!b->graph || b->graph_launches != launches || b->graph_threads != b->threads) {
    drop_graph(b);
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return bfail(b, 100, "nmg_batch_run: capture failed");
    for (int k = 0; k < launches; ++k) launch_run(b);
    if (cudaStreamEndCapture(b->stream, &g) != cudaSuccess || !g) {
      cudaGetLastError();
      return bfail(b, 100, "nmg_batch_run: capture failed");
    }
    cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      return bfail(b, 100, std::string("nmg_batch_run: instantiate: ") + cudaGetErrorString(e));
    }
    b->graph_launches = launches;
    b->graph_threads = b->threads;
  }
  if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) return bfail(b, 100, "nmg_batch_run: graph launch failed");
  return sync_check(b, "nmg_batch_run");
}

int nmg_batch_state(const nmg_batch *b, double *t, int32_t *stage, int64_t *steps, int64_t *rhs, int32_t *done,
                    double *max_dmdt) {
  if (!b) return -1;
  std::vector<nmg::PState> st(b->P);
  // ordered after the batch's own launches, which run on its non-blocking stream
  if (cudaMemcpyAsync(st.data(), b->st.p, sizeof(nmg::PState) * b->P, cudaMemcpyDeviceToHost, b->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess)
    return bfail(const_cast<nmg_batch *>(b), 100, "nmg_batch_state: copy failed");
  for (int p = 0; p < b->P; ++p) {
    if (t) t[p] = st[p].t;
    if (stage) stage[p] = st[p].stage;
    if (steps) steps[p] = st[p].steps;
    if (rhs) rhs[p] = st[p].rhs;
    if (done) done[p] = st[p].done;
    if (max_dmdt) max_dmdt[p] = st[p].maxdmdt;
  }
  return 0;
}

int nmg_batch_set_schedule(nmg_batch *b, int threads, double budget) {
  if (!b || threads < 32 || threads > 1024 || (threads & 31)) return -1;
  b->budget = budget;
  apply_budget(b);
  return set_threads(b, threads);
}

int nmg_batch_autotune(nmg_batch *b, int trial_launches, int *threads_out, double *budget_out) {
  if (!b || trial_launches < 1) return -1;
  // Candidates: CTA size x work budget (in units of the largest particle's
  // cost).  Each is timed on a copy of the state that is restored afterwards,
  // and scored by cost-weighted steps per second.
  const double cmax = std::max_element(b->hdesc.begin(), b->hdesc.end(),
                                       [](const nmg::PDesc &x, const nmg::PDesc &y) { return x.cost < y.cost; })->cost;
  const size_t n3 = 3 * (size_t)b->Ntot;
  nmg::DevBuf<double> save_m, save_k0, save_p1, save_p2, save_hn;
  nmg::DevBuf<nmg::PState> save_st;
  if (save_m.alloc(n3) || save_k0.alloc(n3) || save_p1.alloc(b->Ntot) || save_p2.alloc(b->Ntot) ||
      save_st.alloc(b->P) || (b->hn.p && save_hn.alloc(n3)))
    return bfail(b, 100, "nmg_batch_autotune: allocation failed");
  // Every copy is ordered on the batch's own (non-blocking) stream, so the
  // trial launches on that stream see the saved state and each restore.
  auto d2d = [b](void *dst, const void *src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, b->stream) == cudaSuccess;
  };
  auto copy_state = [&](bool save) {
    bool ok = true;
    if (b->hn.p) ok &= save ? d2d(save_hn.p, b->hn.p, sizeof(double) * n3) : d2d(b->hn.p, save_hn.p, sizeof(double) * n3);
    ok &= save ? d2d(save_m.p, b->m.p, sizeof(double) * n3) : d2d(b->m.p, save_m.p, sizeof(double) * n3);
    ok &= save ? d2d(save_k0.p, b->k0.p, sizeof(double) * n3) : d2d(b->k0.p, save_k0.p, sizeof(double) * n3);
    ok &= save ? d2d(save_p1.p, b->phi1.p, sizeof(double) * b->Ntot) : d2d(b->phi1.p, save_p1.p, sizeof(double) * b->Ntot);
    ok &= save ? d2d(save_p2.p, b->phi2.p, sizeof(double) * b->Ntot) : d2d(b->phi2.p, save_p2.p, sizeof(double) * b->Ntot);
    ok &= save ? d2d(save_st.p, b->st.p, sizeof(nmg::PState) * b->P) : d2d(b->st.p, save_st.p, sizeof(nmg::PState) * b->P);
    return ok;
  };
  auto read_state = [b](std::vector<nmg::PState> &out) {
    return cudaMemcpyAsync(out.data(), b->st.p, sizeof(nmg::PState) * b->P, cudaMemcpyDeviceToHost, b->stream) ==
               cudaSuccess &&
           cudaStreamSynchronize(b->stream) == cudaSuccess;
  };
  std::vector<nmg::PState> st0(b->P), st1(b->P);
  if (!copy_state(true) || !read_state(st0)) return bfail(b, 100, "nmg_batch_autotune: saving the state failed");
  double best = -1.0;
  int best_t = b->threads;
  double best_b = b->budget;
  for (int threads : {128, 256, 512}) {
    for (double f : {0.5, 1.0, 2.0}) {
      if (nmg_batch_set_schedule(b, threads, f * cmax)) continue;
      auto t0 = std::chrono::steady_clock::now();
      for (int k = 0; k < trial_launches; ++k) launch_run(b);
      if (sync_check(b, "nmg_batch_autotune")) {
        copy_state(false);
        break;
      }
      const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (!read_state(st1)) return bfail(b, 100, "nmg_batch_autotune: reading the state failed");
      double work = 0.0;
      for (int p = 0; p < b->P; ++p) work += (double)(st1[p].rhs - st0[p].rhs) * b->hdesc[p].cost;
      const double score = work / sec;
      if (score > best) { best = score; best_t = threads; best_b = f * cmax; }
      if (!copy_state(false)) return bfail(b, 100, "nmg_batch_autotune: restoring the state failed");
    }
  }
  // the last restore (and every copy from the save buffers) completes before
  // they are freed and before the next launch on any stream
  if (cudaStreamSynchronize(b->stream) != cudaSuccess)
    return bfail(b, 100, "nmg_batch_autotune: restoring the state failed");
  int rc = nmg_batch_set_schedule(b, best_t, best_b);
  if (threads_out) *threads_out = best_t;
  if (budget_out) *budget_out = best_b;
  return rc;
}

}  // extern "C"
