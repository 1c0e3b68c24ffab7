// nmg_ts.cu -- device time integrator behind nmg_ts_init / nmg_ts_advance.
//
// Replaces the reference's CVODE timestepper (nsim.ml:1857-2676 callbacks,
// sundials_sp_stubs.c:780-1310 setup and advance): variable-order BDF in
// fixed-leading-coefficient Nordsieck form (orders 1..max_order), modified
// Newton iteration, SPGMR with left preconditioning and ewt scaling, the
// CVODE step/order selection rules and CV_NORMAL(_TSTOP) output.  SUNDIALS is
// not part of the reference tree; the method follows its published
// description (Hindmarsh et al., ACM TOMS 31, 2005).
//
// The state vectors (Nordsieck columns, Krylov basis, work vectors) live on
// the device; every vector operation is a kernel on the handle's stream.  The
// host keeps the scalar step control and reads back one small block of
// scalars per decision (norms, Hessenberg columns).
//
// Jacobian (nmag_lam.py:432-436,684-704; nsim.ml:967-1050,2315-2417):
//   J v = C1 [v x H + m x Hv] + C2 [v x (m x H) + m x (v x H) + m x (m x Hv)],
//   Hv = -c_exch K v / V_i,  with (m, H_total) frozen at the last re-Jacobi.
// Preconditioner: exact inverse of each node's 3x3 block of I - gamma J
// (gamma of the last setup, as the reference's cached KSP).
#include <cmath>
#include <cstring>
#include <vector>

#include "nmg_internal.h"

namespace nmg {
namespace {

constexpr int QMAXB = 5;
constexpr double ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2, ETAMIN = 0.1, ETACF = 0.25;
constexpr double ADDON = 1e-6, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, THRESH = 1.5;
constexpr int SMALL_NST = 10, MXNCF = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, LONG_WAIT = 10, NLS_MAXCOR = 3;
constexpr double CRDOWN = 0.3, DGMAX = 0.3, RDIV = 2.0, CORTES = 0.1;
constexpr int MSBP = 20;
constexpr double SPILS_DGMAX = 0.2, SPILS_DELT = 0.05;
constexpr int SPILS_MSBPRE = 50;
constexpr double UROUND = 2.220446049250313e-16;
constexpr int kRedBlocks = 304;   // two blocks per SM: enough loads in flight for HBM

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- elementwise kernels ----
__global__ void k_lin(int n, double a, const double *__restrict__ x, double b, const double *__restrict__ y,
                      double *__restrict__ z) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = a * x[i] + b * y[i];
}
__global__ void k_scale(int n, double a, double *__restrict__ x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] *= a;
}
// error weights w = 1 / (rtol |y| + atol), and their reciprocals ws (the
// tolerance scale) so that dividing by a weight is a multiplication
__global__ void k_ewt(int n, double rtol, double atol, const double *__restrict__ y, double *__restrict__ w,
                      double *__restrict__ ws) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sc = rtol * fabs(y[i]) + atol;
  w[i] = 1.0 / sc;
  ws[i] = sc;
}
struct ZnPtrs { double *z[QMAXB + 2]; };
// Nordsieck prediction z <- z * Pascal (sign = +1) or its inverse (sign = -1).
// (The order q is a template parameter: with compile-time indices the
// history pointers and values stay in registers.)
template <int Q>
__global__ void k_predict(int n, ZnPtrs zn, int sign) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[Q + 1];
#pragma unroll
  for (int j = 0; j <= Q; ++j) v[j] = zn.z[j][i];
#pragma unroll
  for (int k = 1; k <= Q; ++k)
#pragma unroll
    for (int j = Q; j >= k; --j) v[j - 1] = sign > 0 ? v[j - 1] + v[j] : v[j - 1] - v[j];
#pragma unroll
  for (int j = 0; j < Q; ++j) zn.z[j][i] = v[j];
}
template <int Q>
__global__ void k_rescale(int n, ZnPtrs zn, double eta) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f = eta;
#pragma unroll
  for (int j = 1; j <= Q; ++j) { zn.z[j][i] *= f; f *= eta; }
}
struct Coef { double c[QMAXB + 2]; };
template <int Q>
__global__ void k_complete(int n, ZnPtrs zn, Coef l, const double *__restrict__ acor) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = acor[i];
#pragma unroll
  for (int j = 0; j <= Q; ++j) zn.z[j][i] += l.c[j] * a;
}
// launch K<q>(args...) for the runtime order q in [1, QMAXB]
#define NMG_LAUNCH_Q(K, q, grid, blk, st, ...)                            \
  do {                                                                  \
    switch (q) {                                                        \
      case 1: K<1><<<grid, blk, 0, st>>>(__VA_ARGS__); break;           \
      case 2: K<2><<<grid, blk, 0, st>>>(__VA_ARGS__); break;           \
      case 3: K<3><<<grid, blk, 0, st>>>(__VA_ARGS__); break;           \
      case 4: K<4><<<grid, blk, 0, st>>>(__VA_ARGS__); break;           \
      default: K<5><<<grid, blk, 0, st>>>(__VA_ARGS__); break;          \
    }                                                                   \
  } while (0)
// y(t) = sum_j zn[j] s^j
__global__ void k_interp(int n, int q, ZnPtrs zn, double s, double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = zn.z[q][i];
  for (int j = q - 1; j >= 0; --j) v = zn.z[j][i] + s * v;
  out[i] = v;
}
// Newton residual: tempv = gamma f - (rl1 zn1 + acor)
__global__ void k_newton_res(int n, double gamma, const double *__restrict__ f, double rl1,
                             const double *__restrict__ zn1, const double *__restrict__ acor, double *__restrict__ t) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) t[i] = gamma * f[i] - (rl1 * zn1[i] + acor[i]);
}
// acor += b ; y = zn0 + acor
__global__ void k_newton_upd(int n, const double *__restrict__ b, double *__restrict__ acor,
                             const double *__restrict__ zn0, double *__restrict__ y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = acor[i] + b[i];
  acor[i] = a;
  y[i] = zn0[i] + a;
}
// o = v / w, given ws = 1 / w
__global__ void k_div_ewt(int n, const double *__restrict__ v, const double *__restrict__ ws, double *__restrict__ o) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = v[i] * ws[i];
}
__global__ void k_hub(int n, const double *__restrict__ y, const double *__restrict__ yp, const double *__restrict__ w,
                      double *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = fabs(yp[i]) / (0.1 * fabs(y[i]) + 1.0 / w[i]);
}

// ---- reductions: block partials then one ordered final sum on the host ----
// mode 0: sum (x w)^2 ; mode 1: sum x y ; mode 2: max x
__global__ void k_red(int n, int mode, const double *__restrict__ x, const double *__restrict__ y,
                      double *__restrict__ part) {
  __shared__ double sm[32];
  double acc = 0.0;
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  auto step = [&](double xv, double yv) {
    const double v = xv * yv;
    if (mode == 0) acc += v * v;
    else if (mode == 1) acc += v;
    else acc = fmax(acc, xv);
  };
  for (; i + 3 * stride < n; i += 4 * stride) {   // four loads of each vector in flight, same order
    const double x0 = x[i], x1 = x[i + stride], x2 = x[i + 2 * stride], x3 = x[i + 3 * stride];
    const double y0 = y[i], y1 = y[i + stride], y2 = y[i + 2 * stride], y3 = y[i + 3 * stride];
    step(x0, y0); step(x1, y1); step(x2, y2); step(x3, y3);
  }
  for (; i < n; i += stride) step(x[i], y[i]);
  if (mode == 2) { for (int o = 16; o; o >>= 1) acc = fmax(acc, __shfl_xor_sync(0xffffffffu, acc, o)); }
  else acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = (mode == 2) ? fmax(s, sm[w]) : s + sm[w];
    part[blockIdx.x] = s;
  }
}
// Multi-dot h[k] = V[k] . w for k < nv (Gram-Schmidt), partials per block.
struct VecPtrs { const double *v[32]; };
// NVM: compile-time bound on nv (the accumulators and vector pointers stay
// in registers).
template <int NVM>
__global__ void k_mdot(int n, int nv, VecPtrs V, const double *__restrict__ w, double *__restrict__ part) {
  __shared__ double sm[32][33];
  double acc[NVM];
#pragma unroll
  for (int k = 0; k < NVM; ++k) acc[k] = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double wi = w[i];
#pragma unroll
    for (int k = 0; k < NVM; ++k) if (k < nv) acc[k] += V.v[k][i] * wi;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NVM; ++k) {
    if (k >= nv) break;
    double s = warp_sum(acc[k]);
    if (lane == 0) sm[wid][k] = s;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double s = 0.0;
    for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) s += sm[wv][threadIdx.x];
    part[(size_t)blockIdx.x * 32 + threadIdx.x] = s;
  }
}
// Ordered sum of the multi-dot partials into h (device), one block of 256
// threads: thread (chunk c = tid / 32, value k = tid % 32) adds the partials
// of blocks [c * nblocks / 8, (c + 1) * nblocks / 8) in order, then thread k
// adds the 8 chunk sums in order.
__global__ void __launch_bounds__(256) k_mdot_final(int nblocks, int nv, const double *__restrict__ part,
                                                    double *__restrict__ h, double *__restrict__ hcol, int first) {
  __shared__ double sc[8][32];
  const int k = threadIdx.x & 31, c = threadIdx.x >> 5;
  const int b0 = (int)((long long)c * nblocks / 8), b1 = (int)((long long)(c + 1) * nblocks / 8);
  double s = 0.0;
  if (k < nv) {
#pragma unroll 8
    for (int b = b0; b < b1; ++b) s += part[(size_t)b * 32 + k];
  }
  sc[c][k] = s;
  __syncthreads();
  if (threadIdx.x < nv) {
    double t = 0.0;
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) t += sc[cc][threadIdx.x];
    h[threadIdx.x] = t;
    hcol[threadIdx.x] = first ? t : hcol[threadIdx.x] + t;   // the Hessenberg column, summed over the passes
  }
}
template <int NVM>
__global__ void k_orth(int n, int nv, VecPtrs V, const double *__restrict__ h, double *__restrict__ w) {
  __shared__ double hs[32];
  if (threadIdx.x < nv) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
#pragma unroll
  for (int k = 0; k < NVM; ++k) if (k < nv) s -= hs[k] * V.v[k][i];
  w[i] = s;
}
// x += sum_k c_k V_k with the coefficients passed by value (no host-to-device
// copy, so the host need not wait before reusing its buffer)
struct Coef32 { double c[32]; };
template <int NVM>
__global__ void k_axpy_multi(int n, int nv, VecPtrs V, Coef32 c, double *__restrict__ x) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = x[i];
#pragma unroll
  for (int k = 0; k < NVM; ++k) if (k < nv) s -= (-c.c[k]) * V.v[k][i];
  x[i] = s;
}
void launch_axpy_multi(int n, int nv, const VecPtrs &vp, const Coef32 &c, double *x, cudaStream_t st) {
  const int g = nblk(n, 256);
  if (nv <= 1) k_axpy_multi<1><<<g, 256, 0, st>>>(n, nv, vp, c, x);
  else if (nv <= 2) k_axpy_multi<2><<<g, 256, 0, st>>>(n, nv, vp, c, x);
  else if (nv <= 4) k_axpy_multi<4><<<g, 256, 0, st>>>(n, nv, vp, c, x);
  else if (nv <= 8) k_axpy_multi<8><<<g, 256, 0, st>>>(n, nv, vp, c, x);
  else if (nv <= 16) k_axpy_multi<16><<<g, 256, 0, st>>>(n, nv, vp, c, x);
  else k_axpy_multi<32><<<g, 256, 0, st>>>(n, nv, vp, c, x);
}
// k_orth followed by the block partials of |w|^2, in k_red's grid, order and
// tree (mode 1), so the norm is the same number k_red would give.
template <int NVM>
__global__ void k_orth_norm(int n, int nv, VecPtrs V, const double *__restrict__ h, double *__restrict__ w,
                            double *__restrict__ part) {
  __shared__ double hs[32], sm[32];
  if (threadIdx.x < nv) hs[threadIdx.x] = h[threadIdx.x];
  __syncthreads();
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = w[i];
#pragma unroll
    for (int k = 0; k < NVM; ++k) if (k < nv) s -= hs[k] * V.v[k][i];
    w[i] = s;
    const double v = s * s;
    acc += v;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int wv = 0; wv < (int)(blockDim.x >> 5); ++wv) t = t + sm[wv];
    part[blockIdx.x] = t;
  }
}
void launch_orth_norm(int n, int nv, const VecPtrs &vp, const double *h, double *w, double *part, cudaStream_t st) {
  if (nv <= 1) k_orth_norm<1><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
  else if (nv <= 2) k_orth_norm<2><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
  else if (nv <= 4) k_orth_norm<4><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
  else if (nv <= 8) k_orth_norm<8><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
  else if (nv <= 16) k_orth_norm<16><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
  else k_orth_norm<32><<<kRedBlocks, 256, 0, st>>>(n, nv, vp, h, w, part);
}
// k_orth<NVM> for the smallest NVM >= nv
void launch_orth(int n, int nv, const VecPtrs &vp, const double *h, double *w, cudaStream_t st) {
  const int g = nblk(n, 256);
  if (nv <= 1) k_orth<1><<<g, 256, 0, st>>>(n, nv, vp, h, w);
  else if (nv <= 2) k_orth<2><<<g, 256, 0, st>>>(n, nv, vp, h, w);
  else if (nv <= 4) k_orth<4><<<g, 256, 0, st>>>(n, nv, vp, h, w);
  else if (nv <= 8) k_orth<8><<<g, 256, 0, st>>>(n, nv, vp, h, w);
  else if (nv <= 16) k_orth<16><<<g, 256, 0, st>>>(n, nv, vp, h, w);
  else k_orth<32><<<g, 256, 0, st>>>(n, nv, vp, h, w);
}

// The local terms of dF/dm . w beyond the exchange (Jacobian level >= 1):
// the anisotropy field's derivative (uniaxial, per-node, or polynomial), the
// C3 length term's, and (several materials) the local couplings to the other
// sites of the node.  The reference's Jacobian has none of them
// (nmag_lam.py:665-704: H_exch is its only field derivative).
struct LocalJac {
  int on = 0;
  double C3 = 0.0, K1 = 0.0, anis = 0.0, ax = 0.0, ay = 0.0, az = 1.0;   // one material
  const double *anis_node = nullptr;   // element parameters: per-node anisotropy coefficient
  int nh = 0;                          // polynomial anisotropy field H_d = sum_t c_{t,d} m^{p_t}
  const int32_t *hpow = nullptr;
  const double *hcoef = nullptr;
  const int32_t *site_mat = nullptr;   // several materials: per-site coefficients
  const SiteMat *mt = nullptr;
  const int32_t *site_node = nullptr, *node_ptr = nullptr, *node_sites = nullptr;
  const double *lc = nullptr;          // local coupling table (null: none)
  int n_mats = 0;
};

// dh += dH_local(m) . w (anisotropy; local couplings when tm, the member's
// direction at every site, is given), fw = C3 [(1 - |m|^2) w - 2 (m . w) m]
// (the derivative of C3 (1 - |m|^2) m, nmag_lam.py:417-424).
__device__ __forceinline__ void local_jac(const LocalJac &L, int i, const double *m, const double *w,
                                          const double *tm, double *dh, double *fw) {
  double C3 = L.C3, K1 = L.K1, c = L.anis, ax = L.ax, ay = L.ay, az = L.az;
  bool uni;
  if (L.site_mat) {
    const SiteMat &s = L.mt[L.site_mat[i]];
    C3 = s.C3; K1 = s.K1; c = s.anis; ax = s.ax; ay = s.ay; az = s.az;
    uni = K1 != 0.0;
  } else {
    uni = K1 != 0.0 || L.anis_node;
    if (L.anis_node) c = L.anis_node[i];
  }
  if (uni) {   // H = c am (a - am m), am = a.m
    const double am = (ax * m[0] + ay * m[1]) + az * m[2], aw = (ax * w[0] + ay * w[1]) + az * w[2];
    const double a[3] = {ax, ay, az};
    for (int d = 0; d < 3; ++d) dh[d] += c * ((aw * a[d] - 2.0 * am * aw * m[d]) - am * am * w[d]);
  }
  if (L.nh > 0) {   // d(x^a y^b z^c) = a x^(a-1) y^b z^c dx + ...
    double px[kAnisMaxPow + 1], py[kAnisMaxPow + 1], pz[kAnisMaxPow + 1];
    anis_powers(m[0], m[1], m[2], px, py, pz);
    for (int t = 0; t < L.nh; ++t) {
      const int p = __ldg(L.hpow + t), e0 = p & 15, e1 = (p >> 4) & 15, e2 = (p >> 8) & 15;
      double dm = 0.0;
      if (e0) dm += e0 * px[e0 - 1] * py[e1] * pz[e2] * w[0];
      if (e1) dm += e1 * px[e0] * py[e1 - 1] * pz[e2] * w[1];
      if (e2) dm += e2 * px[e0] * py[e1] * pz[e2 - 1] * w[2];
      for (int d = 0; d < 3; ++d) dh[d] = fma(__ldg(L.hcoef + 3 * t + d), dm, dh[d]);
    }
  }
  if (L.lc && tm) {   // H_lc of site i = sum over the node's other sites s2 of c(X, X2) m_s2
    const int X = L.site_mat[i], nd = L.site_node[i];
    for (int k = L.node_ptr[nd]; k < L.node_ptr[nd + 1]; ++k) {
      const int s2 = L.node_sites[k];
      if (s2 == i) continue;
      const double cc = L.lc[2 * (X * L.n_mats + L.site_mat[s2])];
      const double *w2 = tm + 3 * (size_t)s2;
      dh[0] += cc * w2[0]; dh[1] += cc * w2[1]; dh[2] += cc * w2[2];
    }
  }
  const double mm = (m[0] * m[0] + m[1] * m[1]) + m[2] * m[2], mw = (m[0] * w[0] + m[1] * w[1]) + m[2] * w[2];
  for (int d = 0; d < 3; ++d) fw[d] = C3 * ((1.0 - mm) * w[d] - 2.0 * mw * m[d]);
}

// J v with frozen (mJ, HJ), fused with  w = t - gamma J t  and the block-Jacobi
// preconditioner and the ewt scaling:  out = ewt * P^{-1} (t - gamma J t),
// t = v / ewt (materialised by the caller).  If psolve == 0, out = t - gamma J t;
// raw != 0: out = J t.
struct JvArgs {
  int N, nrep;   // nodes per member, ensemble members (member-major vectors)
  const int32_t *row_ptr, *col_idx, *diag_pos;
  const double *K, *ivol, *mJ, *HJ, *t, *ewt;
  const double *Pinv;   // per node and member: inverse of the 3x3 preconditioner block (row-major)
  const double *pin;    // per-node factor of the Jacobian rows (the pin field) or null
  const int32_t *site_mat;   // several materials: each site's material (null: one material)
  const SiteMat *mt;         //   and the materials' coefficients
  LocalJac L;                // Jacobian level >= 1
  const double *hdv;         // Jacobian level 2: H_demag(t), 3 per node of the potential mesh and member
  int Np;                    //   nodes of that mesh (the site's node: L.site_node)
  double c_exch, C1, C2, gamma, gammap;
  int psolve, scale_out, raw;
  double *out;
};

template <class T>
__device__ __forceinline__ void cross(const T *a, const T *b, T *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// dF = C1 (w x H + m x hv) + C2 (w x (m x H) + m x (w x H + m x hv))
template <class T>
__device__ __forceinline__ void jac_apply(const T *m, const T *H, const T *w, const T *hv, T C1, T C2, T *out) {
  T wxH[3], mxhv[3], mxH[3], t1[3], u[3], t2[3];
  cross(w, H, wxH);
  cross(m, hv, mxhv);
  cross(m, H, mxH);
  cross(w, mxH, t1);
  for (int d = 0; d < 3; ++d) u[d] = wxH[d] + mxhv[d];
  cross(m, u, t2);
  for (int d = 0; d < 3; ++d) out[d] = C1 * (wxH[d] + mxhv[d]) + C2 * (t1[d] + t2[d]);
}

// kLocal: Jacobian level >= 1 (local terms, demag response); the default
// level 0 keeps the lean exchange-only form
template <bool kLocal>
__global__ void k_jv_psolve(JvArgs a) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)a.N * a.nrep) return;
  const int mbr = (int)(g / a.N), i = (int)(g - (long long)mbr * a.N);
  const double *tm = a.t + (size_t)mbr * 3 * a.N;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; ++k) {
    const double *tj = tm + 3 * (size_t)a.col_idx[k];
    double kv = a.K[k];
    s0 += kv * tj[0]; s1 += kv * tj[1]; s2 += kv * tj[2];
  }
  double c_exch = a.c_exch, C1 = a.C1, C2 = a.C2;
  if (a.site_mat) {
    const SiteMat &c = a.mt[a.site_mat[i]];
    c_exch = c.c_exch; C1 = c.C1; C2 = c.C2;
  }
  const double ce = -c_exch * a.ivol[i];
  double hv[3] = {ce * s0, ce * s1, ce * s2};
  const double *m = a.mJ + 3 * (size_t)g, *H = a.HJ + 3 * (size_t)g, *w = a.t + 3 * (size_t)g;
  double fl[3] = {0.0, 0.0, 0.0};
  if constexpr (kLocal) {
    local_jac(a.L, i, m, w, tm, hv, fl);
    if (a.hdv) {
      const int nd = a.L.site_node ? a.L.site_node[i] : i;
      const double *q = a.hdv + 3 * ((size_t)mbr * a.Np + nd);
      hv[0] += q[0]; hv[1] += q[1]; hv[2] += q[2];
    }
  }
  double jw[3];
  jac_apply(m, H, w, hv, C1, C2, jw);
  if constexpr (kLocal) {
    for (int d = 0; d < 3; ++d) jw[d] += fl[d];
  }
  if (a.pin) {
    const double p = a.pin[i];
    jw[0] *= p; jw[1] *= p; jw[2] *= p;
  }
  if (a.raw) {
    for (int d = 0; d < 3; ++d) a.out[3 * (size_t)g + d] = jw[d];
    return;
  }
  double r[3] = {w[0] - a.gamma * jw[0], w[1] - a.gamma * jw[1], w[2] - a.gamma * jw[2]};
  double z[3] = {r[0], r[1], r[2]};
  if (a.psolve) {
    const double *Pi = a.Pinv + 9 * (size_t)g;
    for (int d = 0; d < 3; ++d) z[d] = (Pi[3 * d] * r[0] + Pi[3 * d + 1] * r[1]) + Pi[3 * d + 2] * r[2];
  }
  for (int d = 0; d < 3; ++d) {
    size_t o = 3 * (size_t)g + d;
    a.out[o] = a.scale_out ? a.ewt[o] * z[d] : z[d];
  }
}

// FP32 form of the level-0 J v (jv_precision 1): the same products in FP32
// arithmetic on FP32 copies of the frozen state (mJ, HJ), the preconditioner
// blocks, the exchange matrix and the direction t; out (FP64) as k_jv_psolve's.
// The Newton matrix only needs the accuracy of an approximate Jacobian; its
// FP64 form is bound by the FP64 pipe.
struct Jv32Args {
  int N, nrep;
  const int32_t *row_ptr, *col_idx;
  const float *K, *mJ, *HJ, *t, *Pinv;
  const double *ivol, *ewt, *pin;
  const int32_t *site_mat;
  const SiteMat *mt;
  double c_exch, C1, C2, gamma;
  int psolve, scale_out, raw;
  double *out;
};

__global__ void k_jv32(Jv32Args a) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)a.N * a.nrep) return;
  const int mbr = (int)(g / a.N), i = (int)(g - (long long)mbr * a.N);
  const float *tm = a.t + (size_t)mbr * 3 * a.N;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; ++k) {
    const float *tj = tm + 3 * (size_t)a.col_idx[k];
    const float kv = a.K[k];
    s0 = fmaf(kv, tj[0], s0); s1 = fmaf(kv, tj[1], s1); s2 = fmaf(kv, tj[2], s2);
  }
  double c_exch = a.c_exch, C1 = a.C1, C2 = a.C2;
  if (a.site_mat) {
    const SiteMat &c = a.mt[a.site_mat[i]];
    c_exch = c.c_exch; C1 = c.C1; C2 = c.C2;
  }
  const float ce = (float)(-c_exch * a.ivol[i]);
  const float hv[3] = {ce * s0, ce * s1, ce * s2};
  const float *m = a.mJ + 3 * (size_t)g, *H = a.HJ + 3 * (size_t)g, *w = a.t + 3 * (size_t)g;
  float jw[3];
  jac_apply<float>(m, H, w, hv, (float)C1, (float)C2, jw);
  if (a.pin) {
    const float p = (float)a.pin[i];
    jw[0] *= p; jw[1] *= p; jw[2] *= p;
  }
  if (a.raw) {
    for (int d = 0; d < 3; ++d) a.out[3 * (size_t)g + d] = (double)jw[d];
    return;
  }
  const float gm = (float)a.gamma;
  const float r[3] = {w[0] - gm * jw[0], w[1] - gm * jw[1], w[2] - gm * jw[2]};
  float z[3] = {r[0], r[1], r[2]};
  if (a.psolve) {
    const float *Pi = a.Pinv + 9 * (size_t)g;
    for (int d = 0; d < 3; ++d) z[d] = fmaf(Pi[3 * d], r[0], fmaf(Pi[3 * d + 1], r[1], Pi[3 * d + 2] * r[2]));
  }
  for (int d = 0; d < 3; ++d) {
    const size_t o = 3 * (size_t)g + d;
    a.out[o] = a.scale_out ? a.ewt[o] * (double)z[d] : (double)z[d];
  }
}

// t32 = (float)(v / ewt): the FP32 direction of k_jv32
__global__ void k_div_ewt32(int n, const double *__restrict__ v, const double *__restrict__ ws, float *__restrict__ o) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = (float)(v[i] * ws[i]);
}

__global__ void k_to_f32(long long n, const double *__restrict__ x, float *__restrict__ y) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// The block-Jacobi preconditioner's 3x3 blocks P = I - gamma_p dF/dm (the
// exchange diagonal and the site terms at the setup state mJ, HJ; at
// Jacobian level >= 1 also the local anisotropy and C3 terms), inverted once
// per preconditioner setup: Pinv[9 g + 3 d + c] = (P^-1)_dc.
__global__ void k_pprep(int N, const int32_t *__restrict__ diag_pos, const double *__restrict__ K,
                        const double *__restrict__ vol, const double *__restrict__ mJ, const double *__restrict__ HJ,
                        double c_exch, double C1, double C2, double gammap, double *__restrict__ Pinv, int nrep,
                        const double *__restrict__ pin, const int32_t *__restrict__ site_mat,
                        const SiteMat *__restrict__ mt, LocalJac L, float *__restrict__ Pinv32,
                        float *__restrict__ mJ32, float *__restrict__ HJ32) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)N * nrep) return;
  const int i = (int)(g % N);
  if (site_mat) {   // several materials: the site's own coefficients
    const SiteMat &c = mt[site_mat[i]];
    c_exch = c.c_exch; C1 = c.C1; C2 = c.C2;
  }
  const double kap = -c_exch * K[diag_pos[i]] / vol[i];
  const double pf = pin ? pin[i] : 1.0;
  const double *m = mJ + 3 * (size_t)g, *H = HJ + 3 * (size_t)g;
  double P[3][3];
  for (int c = 0; c < 3; ++c) {
    double e[3] = {0.0, 0.0, 0.0};
    e[c] = 1.0;
    double he[3] = {kap * e[0], kap * e[1], kap * e[2]}, je[3], fe[3] = {0.0, 0.0, 0.0};
    if (L.on) local_jac(L, i, m, e, nullptr, he, fe);
    jac_apply(m, H, e, he, C1, C2, je);
    for (int d = 0; d < 3; ++d) je[d] += fe[d];
    for (int d = 0; d < 3; ++d) P[d][c] = (d == c ? 1.0 : 0.0) - gammap * (pin ? pf * je[d] : je[d]);
  }
  double c00 = P[1][1] * P[2][2] - P[1][2] * P[2][1];
  double c01 = P[1][2] * P[2][0] - P[1][0] * P[2][2];
  double c02 = P[1][0] * P[2][1] - P[1][1] * P[2][0];
  double inv = 1.0 / (P[0][0] * c00 + P[0][1] * c01 + P[0][2] * c02);
  double *o = Pinv + 9 * (size_t)g;
  o[0] = c00 * inv; o[1] = (P[0][2] * P[2][1] - P[0][1] * P[2][2]) * inv; o[2] = (P[0][1] * P[1][2] - P[0][2] * P[1][1]) * inv;
  o[3] = c01 * inv; o[4] = (P[0][0] * P[2][2] - P[0][2] * P[2][0]) * inv; o[5] = (P[0][2] * P[1][0] - P[0][0] * P[1][2]) * inv;
  o[6] = c02 * inv; o[7] = (P[0][1] * P[2][0] - P[0][0] * P[2][1]) * inv; o[8] = (P[0][0] * P[1][1] - P[0][1] * P[1][0]) * inv;
  if (Pinv32) {   // jv_precision 1: the FP32 copies k_jv32 reads
    for (int q = 0; q < 9; ++q) Pinv32[9 * (size_t)g + q] = (float)o[q];
    for (int d = 0; d < 3; ++d) {
      mJ32[3 * (size_t)g + d] = (float)m[d];
      HJ32[3 * (size_t)g + d] = (float)H[d];
    }
  }
}

// Block-Jacobi preconditioner alone: out = ewt * P^{-1} r (r unscaled).
__global__ void k_psolve(long long n3, const double *__restrict__ Pinv, const double *__restrict__ r,
                         const double *__restrict__ ewt, double *__restrict__ out) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (3 * g >= n3) return;
  const double *Pi = Pinv + 9 * (size_t)g, *ri = r + 3 * (size_t)g;
  for (int d = 0; d < 3; ++d) {
    size_t o = 3 * (size_t)g + d;
    out[o] = ewt[o] * ((Pi[3 * d] * ri[0] + Pi[3 * d + 1] * ri[1]) + Pi[3 * d + 2] * ri[2]);
  }
}

}  // namespace

struct Integrator {
  nmg_handle *hd;
  int n, qmax, maxl;
  double rtol, atol;
  DevBuf<double> znbuf, ewt, acor, y, tempv, ftemp, xsol, mJ, HJ, Vbuf, tvec, part, hdev, hcol;
  DevBuf<double> Pinv;   // preconditioner blocks inverted at each setup (9 per node and member)
  // jv_precision 1: FP32 copies of the preconditioner blocks, the frozen
  // state, the exchange matrix, and the direction
  DevBuf<float> Pinv32, mJ32, HJ32, K32, t32;
  DevBuf<double> ewts;   // 1 / ewt
  double *zn[QMAXB + 2];
  std::vector<double *> V;
  double *hpin = nullptr;  // pinned readback
  // CVODE state
  double tn = 0, h = 0, hprime = 0, eta = 1, hscale = 0, etamax = ETAMX1, rl1 = 1, gamma = 0, gammap = 0,
         gamrat = 1, crate = 1, acnrm = 0, nlscoef = CORTES, saved_tq5 = 0, beta0 = 0;
  double tau[QMAXB + 2] = {0}, tq[6] = {0}, l[QMAXB + 1] = {0};
  int q = 1, qprime = 1, qwait = 2, L = 2;
  int64_t nst = 0, nfe = 0, nni = 0, nli = 0, ncfn = 0, netf = 0, nsetups = 0, npe = 0, nps = 0, njv = 0,
          nstlp = 0, nstlpre = 0;
  int jcur = 0, setup_done = 0;
  std::vector<double> Hm, gv, yg;
  int status = 0;  // sticky device / RHS failure

  cudaStream_t s() const { return hd->stream; }
  ZnPtrs znp() const { ZnPtrs z; for (int j = 0; j < QMAXB + 2; ++j) z.z[j] = zn[j]; return z; }

  double wrms(const double *x, const double *w) {
    k_red<<<kRedBlocks, 256, 0, s()>>>(n, 0, x, w, part); ++hd->launches;
    cudaMemcpyAsync(hpin, part.p, sizeof(double) * kRedBlocks, cudaMemcpyDeviceToHost, s());
    if (cudaStreamSynchronize(s()) != cudaSuccess) { status = 100; return 0.0; }
    double acc = 0.0;
    for (int b = 0; b < kRedBlocks; ++b) acc += hpin[b];
    return std::sqrt(acc / n);
  }
  double maxval(const double *x) {
    k_red<<<kRedBlocks, 256, 0, s()>>>(n, 2, x, x, part); ++hd->launches;
    cudaMemcpyAsync(hpin, part.p, sizeof(double) * kRedBlocks, cudaMemcpyDeviceToHost, s());
    if (cudaStreamSynchronize(s()) != cudaSuccess) { status = 100; return 0.0; }
    double mx = 0.0;
    for (int b = 0; b < kRedBlocks; ++b) mx = hpin[b] > mx ? hpin[b] : mx;
    return mx;
  }
  void lin(double a, const double *x, double b, const double *yv, double *z) {
    k_lin<<<nblk(n, 256), 256, 0, s()>>>(n, a, x, b, yv, z); ++hd->launches;
  }
  int rhs(const double *yv, double *f) {
    nfe++;
    int r = rhs_eval(hd, yv, f);
    if (r) status = r;
    return r;
  }
  void set_ewt(const double *yv) { k_ewt<<<nblk(n, 256), 256, 0, s()>>>(n, rtol, atol, yv, ewt, ewts); ++hd->launches; }
};

namespace {

double initial_h(Integrator &I, double tout) {
  const int n = I.n;
  double tdist = std::fabs(tout - I.tn);
  double tround = UROUND * std::fmax(std::fabs(I.tn), std::fabs(tout));
  double hlb = 100.0 * tround;
  k_hub<<<nblk(n, 256), 256, 0, I.s()>>>(n, I.zn[0], I.zn[1], I.ewt, I.tempv); ++I.hd->launches;
  double hub_inv = I.maxval(I.tempv);
  double hub = 0.1 * tdist;
  if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
  double hg = std::sqrt(hlb * hub);
  if (hub < hlb) return hg;
  double hnew = hg;
  int count = 0;
  for (;;) {
    I.lin(hg, I.zn[1], 1.0, I.zn[0], I.y);
    if (I.rhs(I.y, I.tempv)) return hg;
    I.lin(1.0 / hg, I.tempv, -1.0 / hg, I.zn[1], I.tempv);
    double yddnrm = I.wrms(I.tempv, I.ewt);
    hnew = (yddnrm * hub * hub > 2.0) ? std::sqrt(2.0 / yddnrm) : std::sqrt(hg * hub);
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

int psetup(Integrator &I, int jok, const double *ypred) {
  I.npe++;
  if (jok) return 0;
  // The caller evaluated f(ypred) just before, so H_total in the workspace is
  // the field at ypred; the reference re-runs the RHS here (nsim.ml:2338-2348)
  // to get the same field.
  cudaMemcpyAsync(I.mJ.p, ypred, sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
  cudaMemcpyAsync(I.HJ.p, I.hd->ws.h_total.p, sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
  return 1;
}

// The local Jacobian terms of the handle's model (level >= 1), else off.
LocalJac local_jac_args(const nmg_handle *h) {
  LocalJac L;
  if (h->jac_level < 1) return L;
  L.on = 1;
  if (h->pot) {   // several materials
    L.site_mat = h->sites.site_mat.p; L.mt = h->sites.mtab.p;
    L.site_node = h->sites.site_node.p; L.node_ptr = h->sites.node_ptr.p; L.node_sites = h->sites.node_sites.p;
    L.lc = h->sites.lc.p; L.n_mats = h->sites.n_mats;
    return L;
  }
  const nmg_material &mt = h->mat;
  L.C3 = mt.C3; L.K1 = mt.K1; L.anis = mt.anis_coeff;
  L.ax = mt.axis[0]; L.ay = mt.axis[1]; L.az = mt.axis[2];
  if (h->ep.active) {
    L.anis_node = h->ep.anis.p;
    L.ax = h->ep.axis[0]; L.ay = h->ep.axis[1]; L.az = h->ep.axis[2];
  }
  L.nh = h->ap.nh; L.hpow = h->ap.hpow.p; L.hcoef = h->ap.hcoef.p;
  return L;
}

// The FP32 J v form: jv_precision 1 at Jacobian level 0
bool jv_fp32(const nmg_handle *h) { return h->opt.jv_precision == 1 && h->jac_level == 0; }

Jv32Args jv32_base(nmg_handle *h) {
  const Mesh &M = h->mesh;
  Jv32Args a;
  a.N = M.N; a.nrep = h->nrep; a.row_ptr = M.row_ptr; a.col_idx = M.col_idx;
  a.K = a.mJ = a.HJ = a.t = a.Pinv = nullptr;
  a.ivol = M.ivol; a.ewt = nullptr; a.pin = h->pin.p;
  a.site_mat = h->pot ? h->sites.site_mat.p : nullptr;
  a.mt = h->sites.mtab.p;
  a.c_exch = h->mat.exch_coeff; a.C1 = h->mat.C1; a.C2 = h->mat.C2; a.gamma = 0.0;
  a.psolve = 0; a.scale_out = 0; a.raw = 0; a.out = nullptr;
  return a;
}

bool demag_in_jacobian(const nmg_handle *h) {
  return h->jac_level >= 2 && h->opt.do_demag && (h->pot ? h->pot->mesh.nb : h->mesh.nb) > 0;
}

// The handle's part of the J v arguments (no integrator state).
JvArgs jv_base(nmg_handle *h) {
  const Mesh &M = h->mesh;
  JvArgs a;
  a.N = M.N; a.nrep = h->nrep; a.row_ptr = M.row_ptr; a.col_idx = M.col_idx; a.diag_pos = M.diag_pos;
  a.K = h->exch_K(); a.ivol = M.ivol;
  a.pin = h->pin.p;
  a.site_mat = h->pot ? h->sites.site_mat.p : nullptr;
  a.mt = h->sites.mtab.p;
  a.L = local_jac_args(h);
  a.hdv = nullptr;
  a.Np = h->pot ? h->pot->mesh.N : M.N;
  if (!a.L.site_node && h->pot) a.L.site_node = h->sites.site_node.p;   // the demag response's node of a site
  a.c_exch = h->mat.exch_coeff; a.C1 = h->mat.C1; a.C2 = h->mat.C2;
  a.mJ = a.HJ = a.t = a.ewt = a.Pinv = nullptr;
  a.gamma = a.gammap = 0.0; a.psolve = 0; a.scale_out = 0; a.raw = 0; a.out = nullptr;
  return a;
}

JvArgs jv_args(Integrator &I, const double *t, double *out, int psolve) {
  JvArgs a = jv_base(I.hd);
  a.mJ = I.mJ; a.HJ = I.HJ; a.t = t; a.ewt = I.ewt; a.Pinv = I.Pinv;
  a.gamma = I.gamma; a.gammap = I.gammap; a.psolve = psolve; a.scale_out = 1; a.out = out;
  return a;
}

// Gram-Schmidt of w against V[0..nv): two classical passes (CGS2); the
// coefficients stay on the device in hcol.
// Returns true when the second pass also left the block partials of |w|^2
// in I.part (nv <= 32: one chunk).
bool orthogonalise(Integrator &I, int nv, double *w) {
  bool normed = false;
  for (int pass = 0; pass < 2; ++pass) {
    for (int k0 = 0; k0 < nv; k0 += 32) {
      int cnt = nv - k0 < 32 ? nv - k0 : 32;
      VecPtrs vp;
      for (int k = 0; k < cnt; ++k) vp.v[k] = I.V[k0 + k];
      if (cnt <= 1) k_mdot<1><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      else if (cnt <= 2) k_mdot<2><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      else if (cnt <= 4) k_mdot<4><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      else if (cnt <= 8) k_mdot<8><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      else if (cnt <= 16) k_mdot<16><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      else k_mdot<32><<<kRedBlocks, 256, 0, I.s()>>>(I.n, cnt, vp, w, I.part);
      ++I.hd->launches;
      k_mdot_final<<<1, 256, 0, I.s()>>>(kRedBlocks, cnt, I.part, I.hdev.p + k0, I.hcol.p + k0, pass == 0);
      ++I.hd->launches;
    }
    for (int k0 = 0; k0 < nv; k0 += 32) {
      int cnt = nv - k0 < 32 ? nv - k0 : 32;
      VecPtrs vp;
      for (int k = 0; k < cnt; ++k) vp.v[k] = I.V[k0 + k];
      if (pass == 1 && nv <= 32) {
        launch_orth_norm(I.n, cnt, vp, I.hdev.p + k0, w, I.part, I.s());
        normed = true;
      } else {
        launch_orth(I.n, cnt, vp, I.hdev.p + k0, w, I.s());
      }
      ++I.hd->launches;
    }
  }
  return normed;
}

// SPGMR, left preconditioned, scaled by ewt; x = 0 initial guess.
// 0 converged, 2 residual reduced, 1 failure, <0 device error.
int spgmr(Integrator &I, const double *b, double *x, double delta, int *nli_out) {
  const int n = I.n, maxl = I.maxl;
  const Mesh &M = I.hd->mesh;
  const nmg_material &mt = I.hd->mat;
  auto HM = [&](int i, int j) -> double & { return I.Hm[(size_t)i * maxl + j]; };
  *nli_out = 0;
  k_psolve<<<nblk((long long)M.N * I.hd->nrep, 128), 128, 0, I.s()>>>((long long)n, I.Pinv, b, I.ewt, I.V[0]);
  ++I.hd->launches;
  I.nps++;
  double rho = 0.0;  // ||V0||_2 (unweighted)
  {
    k_red<<<kRedBlocks, 256, 0, I.s()>>>(n, 1, I.V[0], I.V[0], I.part); ++I.hd->launches;
    cudaMemcpyAsync(I.hpin, I.part.p, sizeof(double) * kRedBlocks, cudaMemcpyDeviceToHost, I.s());
    if (cudaStreamSynchronize(I.s()) != cudaSuccess) return -1;
    double acc = 0.0;
    for (int bb = 0; bb < kRedBlocks; ++bb) acc += I.hpin[bb];
    rho = std::sqrt(acc);
  }
  cudaMemsetAsync(x, 0, sizeof(double) * n, I.s());
  if (rho <= delta) return 0;
  I.beta0 = rho;
  k_scale<<<nblk(n, 256), 256, 0, I.s()>>>(n, 1.0 / rho, I.V[0]); ++I.hd->launches;
  std::fill(I.yg.begin(), I.yg.end(), 0.0);
  I.yg[0] = rho;
  int converged = 0, kdim = 0;
  for (int l = 0; l < maxl; ++l) {
    // t = V_l / ewt in its own pass: inside the FP64-bound Jv kernel the
    // division would be repeated for every neighbour reference
    if (jv_fp32(I.hd)) {
      if (!I.K32.p) return -1;   // set up with every preconditioner setup (never reached)
      k_div_ewt32<<<nblk(n, 256), 256, 0, I.s()>>>(n, I.V[l], I.ewts, I.t32); ++I.hd->launches;
      Jv32Args a = jv32_base(I.hd);
      a.K = I.K32; a.mJ = I.mJ32; a.HJ = I.HJ32; a.t = I.t32; a.Pinv = I.Pinv32; a.ewt = I.ewt;
      a.gamma = I.gamma; a.psolve = 1; a.scale_out = 1; a.out = I.V[l + 1];
      NMG_PROF_BEGIN(I.hd, 4);
      k_jv32<<<nblk((long long)M.N * I.hd->nrep, 128), 128, 0, I.s()>>>(a);
      ++I.hd->launches;
      NMG_PROF_END(I.hd);
    } else {
      k_div_ewt<<<nblk(n, 256), 256, 0, I.s()>>>(n, I.V[l], I.ewts, I.tvec); ++I.hd->launches;
      JvArgs a = jv_args(I, I.tvec, I.V[l + 1], 1);
      if (demag_in_jacobian(I.hd)) {   // exact Jacobian: the demag field of the direction
        if (demag_response(I.hd, I.tvec)) return -1;
        a.hdv = I.hd->jd.hdv;
      }
      NMG_PROF_BEGIN(I.hd, 4);
      if (a.L.on) k_jv_psolve<true><<<nblk((long long)M.N * I.hd->nrep, 128), 128, 0, I.s()>>>(a);
      else k_jv_psolve<false><<<nblk((long long)M.N * I.hd->nrep, 128), 128, 0, I.s()>>>(a);
      ++I.hd->launches;
      NMG_PROF_END(I.hd);
    }
    I.njv++; I.nps++;
    if (!orthogonalise(I, l + 1, I.V[l + 1])) {
      k_red<<<kRedBlocks, 256, 0, I.s()>>>(n, 1, I.V[l + 1], I.V[l + 1], I.part);
      ++I.hd->launches;
    }
    cudaMemcpyAsync(I.hpin, I.hcol.p, sizeof(double) * (l + 1), cudaMemcpyDeviceToHost, I.s());
    double *hp2 = I.hpin + maxl + 1;
    cudaMemcpyAsync(hp2, I.part.p, sizeof(double) * kRedBlocks, cudaMemcpyDeviceToHost, I.s());
    if (cudaStreamSynchronize(I.s()) != cudaSuccess) return -1;
    for (int k = 0; k <= l; ++k) HM(k, l) = I.hpin[k];
    double acc = 0.0;
    for (int bb = 0; bb < kRedBlocks; ++bb) acc += hp2[bb];
    double hn = std::sqrt(acc);
    HM(l + 1, l) = hn;
    for (int k = 0; k < l; ++k) {
      double c = I.gv[2 * k], sn = I.gv[2 * k + 1];
      double t1 = HM(k, l), t2 = HM(k + 1, l);
      HM(k, l) = c * t1 - sn * t2;
      HM(k + 1, l) = sn * t1 + c * t2;
    }
    double aa = HM(l, l), bb = HM(l + 1, l), c, sn;
    if (bb == 0.0) { c = 1.0; sn = 0.0; }
    else if (std::fabs(bb) > std::fabs(aa)) { double t = aa / bb; sn = -1.0 / std::sqrt(1.0 + t * t); c = -sn * t; }
    else { double t = bb / aa; c = 1.0 / std::sqrt(1.0 + t * t); sn = -c * t; }
    I.gv[2 * l] = c; I.gv[2 * l + 1] = sn;
    HM(l, l) = c * aa - sn * bb;
    HM(l + 1, l) = 0.0;
    I.yg[l + 1] = sn * I.yg[l];
    I.yg[l] = c * I.yg[l];
    rho = std::fabs(I.yg[l + 1]);
    kdim = l + 1;
    if (rho <= delta) { converged = 1; break; }
    if (hn == 0.0) break;
    k_scale<<<nblk(n, 256), 256, 0, I.s()>>>(n, 1.0 / hn, I.V[l + 1]); ++I.hd->launches;
  }
  *nli_out = kdim;
  for (int k = kdim - 1; k >= 0; --k) {
    double sum = I.yg[k];
    for (int j = k + 1; j < kdim; ++j) sum -= HM(k, j) * I.yg[j];
    I.yg[k] = sum / HM(k, k);
  }
  for (int k0 = 0; k0 < kdim; k0 += 32) {
    int cnt = kdim - k0 < 32 ? kdim - k0 : 32;
    VecPtrs vp;
    for (int k = 0; k < cnt; ++k) vp.v[k] = I.V[k0 + k];
    Coef32 c;
    for (int k = 0; k < cnt; ++k) c.c[k] = I.yg[k0 + k];
    launch_axpy_multi(n, cnt, vp, c, x, I.s());   // x -= (-y) V, as the Gram-Schmidt update
    ++I.hd->launches;
  }
  k_div_ewt<<<nblk(n, 256), 256, 0, I.s()>>>(n, x, I.ewts, x); ++I.hd->launches;
  if (converged) return 0;
  return (rho < I.beta0) ? 2 : 1;
}

void predict(Integrator &I) {
  I.tn += I.h;
  NMG_LAUNCH_Q(k_predict, I.q, nblk(I.n, 256), 256, I.s(), I.n, I.znp(), 1); ++I.hd->launches;
}
void restore(Integrator &I, double saved_t) {
  I.tn = saved_t;
  NMG_LAUNCH_Q(k_predict, I.q, nblk(I.n, 256), 256, I.s(), I.n, I.znp(), -1); ++I.hd->launches;
}
void rescale(Integrator &I) {
  NMG_LAUNCH_Q(k_rescale, I.q, nblk(I.n, 256), 256, I.s(), I.n, I.znp(), I.eta); ++I.hd->launches;
  I.h = I.hscale * I.eta;
  I.hprime = I.h;
  I.hscale = I.h;
}

void set_bdf(Integrator &I) {
  const int q = I.q;
  double *l = I.l, *tau = I.tau, h = I.h;
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
  I.tq[2] = std::fabs(A1 / (alpha0 * A2));
  I.tq[5] = std::fabs(A2 * xistar_inv / (l[q] * xi_inv));
  if (I.qwait == 1) {
    if (q > 1) {
      double C = xistar_inv / l[q];
      double A3 = alpha0 + 1.0 / q;
      double A4 = alpha0_hat + xi_inv;
      double Cpinv = (1.0 - A4 + A3) / A3;
      I.tq[1] = std::fabs(C * Cpinv);
    } else {
      I.tq[1] = 1.0;
    }
    hsum += tau[q];
    xi_inv = h / hsum;
    double A5 = alpha0 - 1.0 / (q + 1);
    double A6 = alpha0_hat - xi_inv;
    double Cppinv = (1.0 - A6 + A5) / A2;
    I.tq[3] = std::fabs(Cppinv / (xi_inv * (q + 2) * A5));
  }
  I.tq[4] = I.nlscoef / I.tq[2];
}

// 0 ok, 1 recoverable convergence failure, <0 unrecoverable
int nls(Integrator &I, int nflag_first) {
  const int n = I.n;
  int convfail_bad_j = 0;
  int call_setup = (nflag_first == 2) || (nflag_first == 3) || (I.nst == 0) || (I.nst >= I.nstlp + MSBP) ||
                   (std::fabs(I.gamrat - 1.0) > DGMAX) || !I.setup_done;
  const int convfail_other = !(nflag_first == 1 || nflag_first == 3);
  for (;;) {
    if (I.rhs(I.zn[0], I.ftemp)) return -2;
    if (call_setup) {
      double dgamma = std::fabs(I.gamma / I.gammap - 1.0);
      int jbad = (I.nst == 0) || (I.nst > I.nstlpre + SPILS_MSBPRE) || (convfail_bad_j && dgamma < SPILS_DGMAX) ||
                 (!convfail_bad_j && convfail_other);
      if (!I.setup_done) jbad = 1;
      int jc = psetup(I, !jbad, I.zn[0]);
      if (jc < 0) return -3;
      I.jcur = jc;
      if (jc) I.nstlpre = I.nst;
      I.setup_done = 1;
      I.nsetups++;
      I.crate = 1.0; I.gammap = I.gamma; I.nstlp = I.nst; I.gamrat = 1.0;
      call_setup = 0;
      {
        const Mesh &M = I.hd->mesh;
        const nmg_material &mt = I.hd->mat;
        const bool f32 = jv_fp32(I.hd);
        if (f32) {
          if (!I.K32.p) {   // the FP32 copies, once per integrator
            bool ok = I.K32.alloc(M.nnz) == cudaSuccess && I.Pinv32.alloc(3 * (size_t)I.n) == cudaSuccess;
            for (DevBuf<float> *b : {&I.mJ32, &I.HJ32, &I.t32}) ok = ok && b->alloc(I.n) == cudaSuccess;
            if (!ok) {
              I.hd->last_error = "BDF: cannot allocate the FP32 Jacobian copies";
              return -3;
            }
          }
          k_to_f32<<<nblk((long long)M.nnz, 256), 256, 0, I.s()>>>(M.nnz, I.hd->exch_K(), I.K32);
          ++I.hd->launches;
        }
        k_pprep<<<nblk((long long)M.N * I.hd->nrep, 128), 128, 0, I.s()>>>(
            M.N, M.diag_pos, I.hd->exch_K(), M.vol, I.mJ, I.HJ, mt.exch_coeff, mt.C1, mt.C2, I.gammap, I.Pinv,
            I.hd->nrep, I.hd->pin.p, I.hd->pot ? I.hd->sites.site_mat.p : nullptr, I.hd->sites.mtab.p,
            local_jac_args(I.hd), f32 ? I.Pinv32.p : nullptr, I.mJ32.p, I.HJ32.p);
        ++I.hd->launches;
      }
    }
    cudaMemsetAsync(I.acor.p, 0, sizeof(double) * n, I.s());
    cudaMemcpyAsync(I.y.p, I.zn[0], sizeof(double) * n, cudaMemcpyDeviceToDevice, I.s());
    int m = 0, retry = 0;
    double delp = 0.0, del;
    for (;;) {
      I.nni++;
      k_newton_res<<<nblk(n, 256), 256, 0, I.s()>>>(n, I.gamma, I.ftemp, I.rl1, I.zn[1], I.acor, I.tempv); ++I.hd->launches;
      double deltar = SPILS_DELT * I.tq[4];
      double bnorm = I.wrms(I.tempv, I.ewt);
      if (I.status) return -4;
      int lflag = 0;
      if (bnorm <= deltar) {
        if (m > 0) cudaMemsetAsync(I.tempv.p, 0, sizeof(double) * n, I.s());
      } else {
        int nli = 0;
        int sr = spgmr(I, I.tempv, I.xsol, deltar * std::sqrt((double)n), &nli);
        if (sr < 0) return -4;
        I.nli += nli;
        cudaMemcpyAsync(I.tempv.p, I.xsol.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, I.s());
        if (sr == 1 || (sr == 2 && m > 0)) lflag = 1;
      }
      if (lflag) {
        if (!I.jcur) { convfail_bad_j = 1; call_setup = 1; retry = 1; }
        break;
      }
      del = I.wrms(I.tempv, I.ewt);
      k_newton_upd<<<nblk(n, 256), 256, 0, I.s()>>>(n, I.tempv, I.acor, I.zn[0], I.y); ++I.hd->launches;
      if (m > 0) { double r = del / delp; I.crate = CRDOWN * I.crate > r ? CRDOWN * I.crate : r; }
      double dcon = del * (I.crate < 1.0 ? I.crate : 1.0) / I.tq[4];
      if (dcon <= 1.0) {
        I.acnrm = (m == 0) ? del : I.wrms(I.acor, I.ewt);
        I.jcur = 0;
        return 0;
      }
      ++m;
      if (m == NLS_MAXCOR || (m >= 2 && del > RDIV * delp)) {
        if (!I.jcur) { convfail_bad_j = 1; call_setup = 1; retry = 1; }
        break;
      }
      delp = del;
      if (I.rhs(I.y, I.ftemp)) return -2;
    }
    if (!retry) return 1;
  }
}

void complete_step(Integrator &I) {
  I.nst++;
  for (int i = I.q; i >= 2; --i) I.tau[i] = I.tau[i - 1];
  if (I.q == 1 && I.nst > 1) I.tau[2] = I.tau[1];
  I.tau[1] = I.h;
  Coef c;
  for (int j = 0; j < QMAXB + 2; ++j) c.c[j] = j <= QMAXB ? I.l[j] : 0.0;
  NMG_LAUNCH_Q(k_complete, I.q, nblk(I.n, 256), 256, I.s(), I.n, I.znp(), c, I.acor); ++I.hd->launches;
  I.qwait--;
  if (I.qwait == 1 && I.q != I.qmax) {
    cudaMemcpyAsync(I.zn[I.qmax], I.acor.p, sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
    I.saved_tq5 = I.tq[5];
  }
}

void adjust_order(Integrator &I, int deltaq) {
  const int q = I.q;
  double *l = I.l;
  if (deltaq == 1) {
    for (int i = 0; i <= I.qmax; ++i) l[i] = 0.0;
    l[2] = 1.0;
    double alpha0 = -1.0, alpha1 = 1.0, prod = 1.0, xiold = 1.0, hsum = I.hscale;
    for (int j = 1; j < q; ++j) {
      hsum += I.tau[j + 1];
      double xi = hsum / I.hscale;
      prod *= xi;
      alpha0 -= 1.0 / (j + 1);
      alpha1 += 1.0 / xi;
      for (int i = j + 2; i >= 2; --i) l[i] = l[i] * xiold + l[i - 1];
      xiold = xi;
    }
    double A1 = (-alpha0 - alpha1) / prod;
    I.lin(A1, I.zn[I.qmax], 0.0, I.zn[I.qmax], I.zn[q + 1]);
    for (int j = 2; j <= q; ++j) I.lin(l[j], I.zn[q + 1], 1.0, I.zn[j], I.zn[j]);
  } else if (deltaq == -1) {
    for (int i = 0; i <= I.qmax; ++i) l[i] = 0.0;
    l[2] = 1.0;
    double hsum = 0.0;
    for (int j = 1; j <= q - 2; ++j) {
      hsum += I.tau[j];
      double xi = hsum / I.hscale;
      for (int i = j + 2; i >= 2; --i) l[i] = l[i] * xi + l[i - 1];
    }
    for (int j = 2; j < q; ++j) I.lin(-l[j], I.zn[q], 1.0, I.zn[j], I.zn[j]);
  }
}

void prepare_next_step(Integrator &I, double dsm) {
  if (I.etamax == 1.0) {
    I.qwait = I.qwait > 2 ? I.qwait : 2;
    I.qprime = I.q; I.hprime = I.h; I.eta = 1.0;
    return;
  }
  double etaq = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / I.L) + ADDON);
  if (I.qwait != 0) {
    I.eta = etaq; I.qprime = I.q;
  } else {
    I.qwait = 2;
    double etaqm1 = 0.0, etaqp1 = 0.0;
    if (I.q > 1) {
      double ddn = I.wrms(I.zn[I.q], I.ewt) * I.tq[1];
      etaqm1 = 1.0 / (std::pow(BIAS1 * ddn, 1.0 / I.q) + ADDON);
    }
    if (I.q != I.qmax && I.saved_tq5 != 0.0) {
      double cquot = (I.tq[5] / I.saved_tq5) * std::pow(I.h / I.tau[2], (double)I.L);
      I.lin(-cquot, I.zn[I.qmax], 1.0, I.acor, I.tempv);
      double dup = I.wrms(I.tempv, I.ewt) * I.tq[3];
      etaqp1 = 1.0 / (std::pow(BIAS3 * dup, 1.0 / (I.L + 1)) + ADDON);
    }
    if (etaqm1 > etaq && etaqm1 >= etaqp1) { I.eta = etaqm1; I.qprime = I.q - 1; }
    else if (etaqp1 > etaq) {
      I.eta = etaqp1; I.qprime = I.q + 1;
      cudaMemcpyAsync(I.zn[I.qmax], I.acor.p, sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
    } else { I.eta = etaq; I.qprime = I.q; }
  }
  if (I.eta < THRESH) { I.eta = 1.0; I.qprime = I.q; }
  else if (I.eta > I.etamax) I.eta = I.etamax;
  I.etamax = (I.nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
  I.hprime = I.h * I.eta;
  if (I.qprime < I.q) I.qwait = I.L > 2 ? I.L : 2;
}

int step(Integrator &I) {
  double saved_t = I.tn;
  int ncf = 0, nef = 0, nflag = 1;
  if (I.nst > 0 && (I.hprime != I.h || I.qprime != I.q)) {
    if (I.qprime != I.q) {
      I.hscale = I.h;
      adjust_order(I, I.qprime - I.q);
      I.q = I.qprime; I.L = I.q + 1; I.qwait = I.L;
    }
    I.hscale = I.h;
    I.eta = I.hprime / I.h;
    rescale(I);
  }
  for (;;) {
    predict(I);
    set_bdf(I);
    I.rl1 = 1.0 / I.l[1];
    I.gamma = I.h * I.rl1;
    if (I.nst == 0) I.gammap = I.gamma;
    I.gamrat = (I.nst > 0) ? I.gamma / I.gammap : 1.0;
    int r = nls(I, nflag);
    if (r < 0) { restore(I, saved_t); return 10 - r; }
    if (r == 1) {
      I.ncfn++; ncf++;
      restore(I, saved_t);
      if (ncf == MXNCF) return 4;
      I.etamax = 1.0;
      I.eta = ETACF;
      I.hscale = I.h;
      rescale(I);
      nflag = 2;
      continue;
    }
    double dsm = I.acnrm * I.tq[2];
    if (dsm <= 1.0) {
      complete_step(I);
      prepare_next_step(I, dsm);
      I.etamax = (I.nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
      return 0;
    }
    I.netf++; nef++;
    restore(I, saved_t);
    if (nef == MXNEF) return 5;
    I.etamax = 1.0;
    if (nef <= MXNEF1) {
      I.eta = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / I.L) + ADDON);
      if (I.eta < ETAMIN) I.eta = ETAMIN;
      if (nef >= SMALL_NEF && I.eta > ETAMXF) I.eta = ETAMXF;
      I.hscale = I.h;
      rescale(I);
    } else if (I.q > 1) {
      I.eta = ETAMIN;
      I.hscale = I.h;
      adjust_order(I, -1);
      I.L = I.q; I.q--; I.qwait = I.L;
      rescale(I);
    } else {
      I.eta = ETAMIN;
      I.h *= I.eta; I.hscale = I.h; I.hprime = I.h;
      I.qwait = LONG_WAIT;
      if (I.rhs(I.zn[0], I.tempv)) return 12;
      I.lin(I.h, I.tempv, 0.0, I.tempv, I.zn[1]);
    }
    nflag = 3;
  }
}

void interpolate(Integrator &I, double t, double *out) {
  double sv = (t - I.tn) / I.h;
  k_interp<<<nblk(I.n, 256), 256, 0, I.s()>>>(I.n, I.q, I.znp(), sv, out); ++I.hd->launches;
}

}  // namespace

Integrator *ts_create(nmg_handle *h, int qmax, int maxl, double rtol, double atol) {
  Integrator *I = new Integrator();
  I->hd = h;
  I->n = 3 * h->mesh.N * h->nrep;
  I->qmax = qmax < 1 ? 1 : (qmax > QMAXB ? QMAXB : qmax);
  I->maxl = maxl < 1 ? 5 : maxl;
  I->rtol = rtol; I->atol = atol;
  const size_t n = I->n;
  bool ok = I->znbuf.alloc(n * (I->qmax + 2)) == cudaSuccess;
  for (DevBuf<double> *b : {&I->ewt, &I->ewts, &I->acor, &I->y, &I->tempv, &I->ftemp, &I->xsol, &I->mJ, &I->HJ, &I->tvec})
    ok = ok && b->alloc(n) == cudaSuccess;
  ok = ok && I->Vbuf.alloc(n * (I->maxl + 1)) == cudaSuccess;
  ok = ok && I->Pinv.alloc(3 * n) == cudaSuccess;
  ok = ok && I->part.alloc(32 * kRedBlocks) == cudaSuccess;
  ok = ok && I->hdev.alloc(I->maxl + 64) == cudaSuccess;
  ok = ok && I->hcol.alloc(I->maxl + 64) == cudaSuccess;
  ok = ok && cudaMallocHost(&I->hpin, sizeof(double) * (I->maxl + 1 + kRedBlocks + 64)) == cudaSuccess;
  if (!ok) { ts_destroy(I); return nullptr; }
  for (int j = 0; j < QMAXB + 2; ++j) I->zn[j] = j <= I->qmax + 1 ? I->znbuf.p + n * j : nullptr;
  I->V.resize(I->maxl + 1);
  for (int j = 0; j <= I->maxl; ++j) I->V[j] = I->Vbuf.p + n * j;
  I->Hm.assign((size_t)(I->maxl + 1) * I->maxl, 0.0);
  I->gv.assign(2 * (size_t)I->maxl, 0.0);
  I->yg.assign(I->maxl + 1, 0.0);
  return I;
}

bool ts_matches(const Integrator *I, int qmax, int maxl) { return I->qmax == qmax && I->maxl == maxl; }
// The next Newton iteration sets up its preconditioner afresh (the Jacobian's level changed).
void ts_invalidate_setup(Integrator *I) {
  if (I) I->setup_done = 0;
}
void ts_set_tolerances(Integrator *I, double rtol, double atol) { I->rtol = rtol; I->atol = atol; }

void ts_destroy(Integrator *I) {
  if (!I) return;
  if (I->hpin) cudaFreeHost(I->hpin);
  delete I;
}

int ts_init(nmg_handle *h, double t0) {
  Integrator &I = *h->ts;
  I.tn = t0; I.q = 1; I.L = 2; I.qwait = I.L; I.qprime = 1;
  I.nst = I.nfe = I.nni = I.nli = I.ncfn = I.netf = I.nsetups = I.npe = I.nps = I.njv = 0;
  I.nstlp = I.nstlpre = 0;
  I.etamax = ETAMX1; I.h = 0.0; I.hprime = 0.0; I.nlscoef = CORTES;
  I.setup_done = 0; I.jcur = 0; I.status = 0; I.saved_tq5 = 0.0;
  for (int i = 0; i < QMAXB + 2; ++i) I.tau[i] = 0.0;
  for (int i = 0; i < 6; ++i) I.tq[i] = 0.0;
  cudaMemcpyAsync(I.zn[0], h->ws.m.p, sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
  for (int j = 1; j <= I.qmax + 1; ++j) cudaMemsetAsync(I.zn[j], 0, sizeof(double) * I.n, I.s());
  I.set_ewt(I.zn[0]);
  if (I.rhs(I.zn[0], I.zn[1])) return I.status ? I.status : 100;
  int rc = check_device_error(h, "ts_init");
  h->ts_ready = rc == 0;
  return rc;
}

int ts_advance(nmg_handle *h, double tout, int exact_tstop, int64_t max_steps, double *t_reached,
               nmg_ts_stats *st) {
  Integrator &I = *h->ts;
  int rc = 0;
  if (I.nst == 0 && I.h == 0.0) {
    double h0 = initial_h(I, tout);
    if (I.status) return I.status;
    if (exact_tstop && (I.tn + h0 - tout) * h0 > 0.0) h0 = (tout - I.tn) * (1.0 - 4.0 * UROUND);
    I.h = h0; I.hprime = h0; I.hscale = h0; I.qprime = I.q;
    k_scale<<<nblk(I.n, 256), 256, 0, I.s()>>>(I.n, h0, I.zn[1]); ++I.hd->launches;
  }
  int64_t taken = 0;
  double troundoff = 100.0 * UROUND * (std::fabs(I.tn) + std::fabs(I.h));
  for (;;) {
    if (!exact_tstop && (I.tn - tout) * I.h >= 0.0) { interpolate(I, tout, h->ws.m); *t_reached = tout; break; }
    if (exact_tstop && std::fabs(I.tn - tout) <= troundoff) { interpolate(I, tout, h->ws.m); *t_reached = tout; break; }
    if (max_steps >= 0 && taken >= max_steps) {
      cudaMemcpyAsync(h->ws.m.p, I.zn[0], sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
      *t_reached = I.tn;
      break;
    }
    if (exact_tstop && (I.tn + I.hprime - tout) * I.hprime > 0.0) I.hprime = (tout - I.tn) * (1.0 - 4.0 * UROUND);
    I.set_ewt(I.zn[0]);
    int r = step(I);
    if (r) {
      rc = r;
      cudaMemcpyAsync(h->ws.m.p, I.zn[0], sizeof(double) * I.n, cudaMemcpyDeviceToDevice, I.s());
      *t_reached = I.tn;
      h->last_error = "time integration failed (code " + std::to_string(r) + ")";
      break;
    }
    ++taken;
    troundoff = 100.0 * UROUND * (std::fabs(I.tn) + std::fabs(I.h));
  }
  int de = check_device_error(h, "ts_advance");
  if (!rc && de) rc = de;
  if (st) {
    st->nst = I.nst; st->nfe = I.nfe; st->nni = I.nni; st->nli = I.nli; st->ncfn = I.ncfn; st->netf = I.netf;
    st->npe = I.npe; st->nps = I.nps; st->njv = I.njv; st->nje = I.nsetups;
    st->hcur = I.h; st->tcur = I.tn; st->qcur = I.q;
    int it[2] = {0, 0};
    cudaMemcpyAsync(it, h->ws.iters.p, sizeof(it), cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    st->last_cg_iters_nbc = it[0]; st->last_cg_iters_dbc = it[1];
  }
  return rc;
}

// Classical RK4 with fixed dt on device vectors (differentiation form forward).
int rk4_device(nmg_handle *h, double *d_m, double dt, int nsteps) {
  const int n = 3 * h->mesh.N * h->nrep;
  DevBuf<double> buf;
  if (buf.alloc(5 * (size_t)n)) return 100;
  double *k1 = buf.p, *k2 = k1 + n, *k3 = k2 + n, *k4 = k3 + n, *y = k4 + n;
  cudaStream_t s = h->stream;
  for (int st = 0; st < nsteps; ++st) {
    if (rhs_eval(h, d_m, k1)) return 100;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, d_m, 0.5 * dt, k1, y); ++h->launches;
    if (rhs_eval(h, y, k2)) return 100;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, d_m, 0.5 * dt, k2, y); ++h->launches;
    if (rhs_eval(h, y, k3)) return 100;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, d_m, dt, k3, y); ++h->launches;
    if (rhs_eval(h, y, k4)) return 100;
    // m += dt/6 (k1 + 2 k2 + 2 k3 + k4)
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, k1, 2.0, k2, y); ++h->launches;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, y, 2.0, k3, y); ++h->launches;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, y, 1.0, k4, y); ++h->launches;
    k_lin<<<nblk(n, 256), 256, 0, s>>>(n, 1.0, d_m, dt / 6.0, y, d_m); ++h->launches;
  }
  return check_device_error(h, "rk4");
}

// d_out = J(d_m) d_v with the handle's Jacobian level: the RHS at d_m gives
// H_total (the frozen field of the Newton matrix), then the fused J v kernel
// without the preconditioner.
int jacobian_apply(nmg_handle *h, const double *d_m, const double *d_v, double *d_out) {
  if (rhs_eval(h, d_m, nullptr)) return 100;
  if (jv_fp32(h)) {   // the FP32 form on FP32 copies, as the integrator forms them
    const long long n = 3LL * h->mesh.N * h->nrep, nnz = h->mesh.nnz;
    DevBuf<float> buf;
    if (buf.alloc((size_t)(nnz + 3 * n)) != cudaSuccess) return 100;
    float *K32 = buf.p, *m32 = K32 + nnz, *H32 = m32 + n, *t32 = H32 + n;
    k_to_f32<<<nblk(nnz, 256), 256, 0, h->stream>>>(nnz, h->exch_K(), K32);
    k_to_f32<<<nblk(n, 256), 256, 0, h->stream>>>(n, d_m, m32);
    k_to_f32<<<nblk(n, 256), 256, 0, h->stream>>>(n, h->ws.h_total, H32);
    k_to_f32<<<nblk(n, 256), 256, 0, h->stream>>>(n, d_v, t32);
    Jv32Args a = jv32_base(h);
    a.K = K32; a.mJ = m32; a.HJ = H32; a.t = t32; a.raw = 1; a.out = d_out;
    k_jv32<<<nblk((long long)h->mesh.N * h->nrep, 128), 128, 0, h->stream>>>(a);
    h->launches += 5;
    if (cudaGetLastError() != cudaSuccess) return 100;
    return check_device_error(h, "nmg_jacobian_apply");   // synchronises before buf is freed
  }
  JvArgs a = jv_base(h);
  a.mJ = d_m; a.HJ = h->ws.h_total; a.t = d_v; a.raw = 1; a.out = d_out;
  if (demag_in_jacobian(h)) {
    if (demag_response(h, d_v)) return 100;
    a.hdv = h->jd.hdv;
  }
  if (a.L.on) k_jv_psolve<true><<<nblk((long long)h->mesh.N * h->nrep, 128), 128, 0, h->stream>>>(a);
  else k_jv_psolve<false><<<nblk((long long)h->mesh.N * h->nrep, 128), 128, 0, h->stream>>>(a);
  ++h->launches;
  if (cudaGetLastError() != cudaSuccess) return 100;
  return check_device_error(h, "nmg_jacobian_apply");
}

}  // namespace nmg
