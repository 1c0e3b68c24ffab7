// rhs_kernels.cu -- the LLG right-hand side on the device.
//
// Replaces the reference's RHS program update_dmdt (interface/nmag/nmag_lam.py
// :784-795): set_H_demag (:740-760; PETSc MatMult + two KSPSolves + dense BEM
// MatMult), set_H_exch (:734-739), the site-wise anisotropy, H_total and LLG
// local equations (:417-430,503,635-650; generated C run by fem_stubs.c:42-144).
//
// Kernels:
//   k_div          rho = -Ms * sum_k D(i,k) . m_k                 (op_div_m + SCALE -1)
//   k_cg3          persistent cooperative Jacobi-PCG (single-reduction form), bounded barriers
//   k_gather_b     phi1b = phi1[node_of_b]                          (PULL-FEM)
//   k_gemv_*       phi2b = BEM phi1b, row-major warp segments + ordered row sum
//   k_dbc_rhs      rhs = -K_IB phi2b (interior), phi2b (boundary)  (op_load_DBC)
//   k_heff_llg     H_exch (K SpMV), H_demag (G SpMV on phi1+phi2), H_anis,
//                  H_total and dm/dt fused in one node kernel (CFBOX = / V_i)
//   k_anis_poly    H_anis from the polynomial form of a general anisotropy
//                  energy (uniaxial K2, cubic, user functions), before k_heff_llg
//   k_stt_dmdc     spin-transfer dm_dcurrent = (J . grad) m, before k_heff_llg
#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <cstring>
#include <utility>

#include "nmg_internal.h"

namespace nmg {
namespace {

constexpr unsigned long long kBarrierSpinLimit = 1ull << 24;  // ~1-2 s with nanosleep
constexpr int kCGThreads = 256;

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum each of NV values over the warp with recursive halving (31 shuffles for
// NV = 32): afterwards lane L holds the total of value L >> (5 - log2 NV).
template <typename T, int NV>
__device__ __forceinline__ T warp_transpose_sum(T (&v)[NV]) {
  const int lane = threadIdx.x & 31;
  int n = NV;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (n > 1) {
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int i = 0; i < NV / 2; ++i) {
        if (i >= n / 2) break;
        const T send = up ? v[i] : v[i + n / 2];
        const T keep = up ? v[i + n / 2] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
      n >>= 1;
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    }
  }
  return v[0];
}

// Shape of a block reduction of NV values: transpose groups of Q values
// (a power of two, at most 32), G groups; lane L ends with value L >> SH of
// each group.
template <int NV>
struct RedShape {
  static constexpr int Q = NV > 16 ? 32 : (NV > 8 ? 16 : (NV > 4 ? 8 : (NV > 2 ? 4 : (NV > 1 ? 2 : 1))));
  static constexpr int G = (NV + Q - 1) / Q;
  static constexpr int SH = Q == 32 ? 0 : (Q == 16 ? 1 : (Q == 8 ? 2 : (Q == 4 ? 3 : (Q == 2 ? 4 : 5))));
  static constexpr int W = G * Q;   // per-warp stride of the scratch
};

// Block-wide sum of NV values in a fixed order; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = warp_sum(v[j]);
    if (lane == 0) smem[wid * NV + j] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += smem[w * NV + j];
      v[j] = s;
    }
  }
  __syncthreads();
}

// Block sum of NV values per thread in a fixed order, the totals written as
// double to out[j * stride], j < NV, by threads 0..NV-1 (out may be global).  Each warp
// reduces its lanes with transpose sums (one shuffle-add per value per
// stage at the widest, against five for a butterfly per value), then
// thread j adds value j over the warps.  smem: (kCGThreads/32) x W values.
template <typename T, int NV>
__device__ __forceinline__ void block_reduce_out(const T (&v)[NV], T *smem, double *out, int stride = 1) {
  using S = RedShape<NV>;
  constexpr int NW = kCGThreads / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int g = 0; g < S::G; ++g) {
    T w[S::Q];
#pragma unroll
    for (int i = 0; i < S::Q; ++i) w[i] = (g * S::Q + i < NV) ? v[g * S::Q + i] : T(0);
    const T t = warp_transpose_sum<T, S::Q>(w);
    const int j = g * S::Q + (lane >> S::SH);
    if ((lane & ((1 << S::SH) - 1)) == 0 && j < NV) smem[wid * S::W + j] = t;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    T t = T(0);
#pragma unroll
    for (int w = 0; w < NW; ++w) t += smem[w * S::W + threadIdx.x];
    out[(size_t)threadIdx.x * stride] = (double)t;
  }
}

// res[j] = sum over the grid's blocks b of slot[j * gridDim.x + b] (block
// partials stored value-major, so a warp's loads of one value are
// contiguous), j < NV, in a fixed order, identical in every block: warp w
// takes the values j = w, w + 8, ...; its lanes take blocks lane, lane + 32,
// ... (all of a lane's loads issued together), then one transpose sum per
// warp.  res: shared.
template <int NV>
__device__ __forceinline__ void grid_total(const double *slot, double *res) {
  constexpr int NW = kCGThreads / 32;
  constexpr int JV = (NV + NW - 1) / NW;
  using S = RedShape<JV>;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double t[S::Q];
#pragma unroll
  for (int q = 0; q < S::Q; ++q) t[q] = 0.0;
#pragma unroll 4
  for (unsigned b = lane; b < gridDim.x; b += 32) {
#pragma unroll
    for (int q = 0; q < JV; ++q) {
      const int j = wid + q * NW;
      if (j < NV) t[q] += __ldcg(slot + (size_t)j * gridDim.x + b);
    }
  }
  const double tot = warp_transpose_sum<double, S::Q>(t);
  const int q = lane >> S::SH, j = wid + q * NW;
  if ((lane & ((1 << S::SH) - 1)) == 0 && q < JV && j < NV) res[j] = tot;
  __syncthreads();
}

struct CGArgs {
  int N, mode;  // mode 0: K (Neumann, constant null space projected); 1: K_II (+) I_B
  const int32_t *row_ptr, *col_idx, *b_of_node;
  const double *K, *dinv, *b;
  double *x, *r, *z, *p, *q, *red;
  unsigned *bar;
  int *err, *iters;
  double rtol, atol;
  int maxits;
  double *w;          // A u (single-reduction CG)
  unsigned *flags;    // barrier counter (word 0)
  double *tot;        // unused
  // solver ordering: row r of the solve is node perm[r]; CSR in that order
  const int32_t *perm, *prow, *pcol, *pbnd;   // pbnd[r]: node perm[r] is a boundary node
  const double *pK;
  double *xperm;      // current iterate in solver order (published for the SpMV)
  // two-level preconditioner (mode 0): aggregates of kAgg consecutive rows
  int coarse, nc;
  const double *ainv; // nc x nc inverse of the (regularised) aggregated operator
  double *rc;         // restricted residual, nc
  // mixed-precision CG: FP32 copies for the inner iterations
  const float *ainv32;
  float *rc32, *z32;  // coarse residual (nc x MB), published inner direction (N x MB)
  float *rw32;        // R w of every aggregate (nc x MB), published with the inner dot products
  float eta;          // inner relative tolerance
  // the mixed-precision CG's rows as each block keeps them in shared memory:
  // the columns inside the block's row range first (mmid[r] of them), values
  // with the Dirichlet rows' boundary columns zeroed for mode 1
  const int32_t *mcol, *mmid;
  const double *mK0, *mK1;
  const float *mK32_0, *mK32_1;
  int max_outer;      // FP64 refinement steps
  int local_sweeps;   // mixed-precision CG: damped Jacobi sweeps on the block's own rows (1: plain Jacobi)
};
constexpr int kAgg = 64;   // rows per aggregate (4 aggregates per 256-row block)
// float4 groups of the coarse vectors (nc x MB floats) per thread of the
// mixed-precision CG: nc * kChunk <= kRwPer * 4 * kCGThreads, i.e. up to 640
// aggregates (40,960 nodes; its one-block-per-SM grid holds 38,912 rows)
constexpr int kRwPer = 5;

// ---- single-reduction CG on a counter barrier ----
constexpr int kCG2MaxRed = 12 * kChunk;   // widest fused reduction (projection dots, b.b and sum b per member)

// gpu-scope acquire load
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Counter barrier: thread 0 of every block does a gpu-scope release add on
// one word and waits (acquire) until it reaches epoch * nblocks.  About 1.2 us
// on GB300 at 121 blocks, against 5.6 us for the gather-at-block-0 barrier.
__device__ __forceinline__ bool arrive_wait(const CGArgs &a, unsigned epoch) {
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned *cnt = a.flags;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(cnt) : "memory");
    const unsigned target = epoch * gridDim.x;
    unsigned long long spins = 0;
    while (ld_acquire_gpu(cnt) < target) {
      if (++spins > kBarrierSpinLimit || (*(volatile int *)a.err & ERR_BARRIER)) { atomicOr(a.err, ERR_BARRIER); break; }
    }
  }
  __syncthreads();
  return !(*(volatile int *)a.err & ERR_BARRIER);
}

// arrive_wait in two halves, so that a block can work between its arrival
// and the wait (same counter, same spin limit and error flag).
__device__ __forceinline__ void arrive(const CGArgs &a) {
  __syncthreads();
  if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(a.flags) : "memory");
}
__device__ __forceinline__ bool wait_epoch(const CGArgs &a, unsigned epoch) {
  if (threadIdx.x == 0) {
    const unsigned target = epoch * gridDim.x;
    unsigned long long spins = 0;
    while (ld_acquire_gpu(a.flags) < target) {
      if (++spins > kBarrierSpinLimit || (*(volatile int *)a.err & ERR_BARRIER)) { atomicOr(a.err, ERR_BARRIER); break; }
    }
  }
  __syncthreads();
  return !(*(volatile int *)a.err & ERR_BARRIER);
}

// Reduction fused with the counter barrier: partials double-buffered by
// epoch parity; after the barrier every block sums all partials in block
// order (deterministic, identical in every block).  smem: block_reduce_out
// scratch ((kCGThreads/32) x RedShape<NV>::W doubles) followed by NV totals.
template <int NV>
__device__ __forceinline__ bool reduce_all(const CGArgs &a, unsigned epoch, double (&v)[NV], double *smem,
                                           double (&out)[NV]) {
  double *slot = a.red + (size_t)(epoch & 1) * gridDim.x * kCG2MaxRed;
  block_reduce_out<double, NV>(v, smem, slot + blockIdx.x, gridDim.x);
  if (!arrive_wait(a, epoch)) return false;
  double *res = smem + (kCGThreads / 32) * RedShape<NV>::W;
  grid_total<NV>(slot, res);
#pragma unroll
  for (int j = 0; j < NV; ++j) out[j] = res[j];
  __syncthreads();
  return true;
}

// reduce_all with the totals left in shared memory (res[0..NV)) instead of
// registers: the ensemble CG keeps its per-member values there.
template <int NV>
__device__ __forceinline__ bool reduce_all_to(const CGArgs &a, unsigned epoch, double (&v)[NV], double *smem,
                                              double *res) {
  double *slot = a.red + (size_t)(epoch & 1) * gridDim.x * kCG2MaxRed;
  block_reduce_out<double, NV>(v, smem, slot + blockIdx.x, gridDim.x);
  if (!arrive_wait(a, epoch)) return false;
  grid_total<NV>(slot, res);
  return true;
}

// Jacobi-preconditioned CG in the single-reduction (Chronopoulos-Gear) form,
// one row per thread, the block's CSR rows (Dirichlet-masked columns zeroed)
// resident in shared memory; each iteration gathers only the neighbours' u
// from L2.  Stopping rule ||r||_2 <= max(rtol ||b - mean||_2, atol).
//
// Initial guess: the solution is linear in b, so b is projected (least
// squares) onto the span of the last kBasis right-hand sides of this solve
// kind, and x starts from the same combination of their solutions.  The dots
// b.b_j come with the first reduction and also update the Gram matrix; every
// block solves the small system identically.  With an empty basis the
// previous solution is the start, like the reference's initial_guess_nonzero.
constexpr int kBasis = kBasisMax;
constexpr int kCGSlots = 4;   // warm-start bases: 0/1 Neumann/Dirichlet, 2/3 the adjoint solves

struct CGBasis {
  double *b, *x;   // kBasis x N right-hand sides and solutions
  double *gram;    // kBasis x kBasis
  int *ring;       // {count, head}
  GramLDL *ldl;    // mixed-precision CG: the factor of each member's Gram system (null: none)
};

// Least squares for c: (G + eps diag G) c = v, one warp (every lane calls;
// lane i < n owns row i of L): LDL^T factorisation, column by column, with
// the rows of a column in parallel lanes; a direction whose pivot collapses
// (nearly dependent right-hand sides) gets c = 0.  Each pivot's reciprocal
// is formed once and the substitutions multiply: the dependent chain is n
// reciprocals instead of ~n^2/2 FP64 divisions in one thread.  sD: kBasis
// doubles of shared scratch for this warp (the pivots); c (shared or
// global) receives c[0..n) from lanes 0..n-1.
// The warp's LDL^T factorisation of (G + eps diag G): lane i keeps row i of
// the unit lower factor in L, rd = 1 / D_i (0: dropped direction), `on` the
// kept directions.  sD: kBasis doubles of shared scratch (the pivots).
__device__ __forceinline__ void small_factor_warp(int n, const double *G, double *sD, double (&L)[kBasis],
                                                  double &rd, unsigned &on) {
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  rd = 0.0;
  on = 0u;
#pragma unroll
  for (int j = 0; j < kBasis; ++j) L[j] = 0.0;
#pragma unroll
  for (int j = 0; j < kBasis; ++j) {
    if (j >= n) break;
    double s = lane < n ? G[lane * kBasis + j] : 0.0;
    if (lane == j) s *= 1.0 + 1e-12;
#pragma unroll
    for (int k = 0; k < kBasis; ++k) {
      if (k >= j) break;
      const double ljk = __shfl_sync(full, L[k], j);
      if ((on >> k) & 1u) s -= (L[k] * sD[k]) * ljk;
    }
    const double sjj = __shfl_sync(full, s, j);
    const bool keep = sjj > 1e-14 * G[j * kBasis + j];
    const double r = keep ? 1.0 / sjj : 0.0;
    __syncwarp();
    if (lane == 0) sD[j] = keep ? sjj : 1.0;
    __syncwarp();
    if (keep) on |= 1u << j;
    if (lane == j) rd = r;
    if (lane > j) L[j] = s * r;
  }
}

// c = (G + eps diag G)^-1 v from the factor: L z = v, y = z / D, L^T c = y.
__device__ __forceinline__ void small_subst_warp(int n, const double (&L)[kBasis], double rd, unsigned on,
                                                 const double *v, double *c) {
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  double z = lane < n ? v[lane] : 0.0;
#pragma unroll
  for (int k = 0; k < kBasis; ++k) {
    if (k >= n) break;
    const double zk = __shfl_sync(full, z, k);
    if (lane > k && ((on >> k) & 1u)) z -= L[k] * zk;
  }
  double ci = z * rd;
  // L^T c = y, descending: lane i takes L_ki from lane k's row
#pragma unroll
  for (int k = kBasis - 1; k >= 0; --k) {
    if (k >= n) continue;
    if (lane == k && !((on >> k) & 1u)) ci = 0.0;
    const double ck = __shfl_sync(full, ci, k);
#pragma unroll
    for (int i = 0; i < kBasis; ++i) {
      if (i >= k) break;
      const double lki = __shfl_sync(full, L[i], k);
      if (lane == i) ci -= lki * ck;
    }
  }
  if (lane < n) c[lane] = ((on >> lane) & 1u) ? ci : 0.0;
}

__device__ void small_solve_warp(int n, const double *G, const double *v, double *c, double *sD) {
  double L[kBasis], rd;
  unsigned on;
  small_factor_warp(n, G, sD, L, rd, on);
  small_subst_warp(n, L, rd, on, v, c);
}

// The mixed-precision CG's warm-start factor of each member's Gram system,
// formed on the auxiliary stream after a solve for the next solve of that
// basis (which then only substitutes: the same arithmetic as the whole warp
// solve, off its critical path).  Warp m: member m.
__global__ void __launch_bounds__(32 * kChunk) k_gram_factor(CGBasis B, int nm) {
  __shared__ double sD[kChunk][kBasis];
  const int m = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (m >= nm) return;
  const int n = B.ring[2 * m];
  double L[kBasis], rd;
  unsigned on;
  small_factor_warp(n, B.gram + (size_t)m * kBasis * kBasis, sD[m], L, rd, on);
  GramLDL &f = B.ldl[m];
  if (lane < kBasis) {
#pragma unroll
    for (int j = 0; j < kBasis; ++j) f.L[lane * kBasis + j] = L[j];
    f.rd[lane] = rd;
  }
  if (lane == 0) { f.on = on; f.n = n; }
}

__global__ void __launch_bounds__(kCGThreads, 4) k_cg3(CGArgs a, int nnz_cap, CGBasis B) {
  extern __shared__ double dyn[];
  __shared__ double smem[kCGThreads / 32 * RedShape<kBasis + 1>::W + kBasis + 1];   // reduce_all scratch + totals
  __shared__ double sc[kBasis + 4];
  __shared__ double sagg[2 * (kCGThreads / kAgg)], sec[kCGThreads / kAgg];
  double *sK = dyn;
  int *sC = reinterpret_cast<int *>(sK + nnz_cap);
  const int row0 = blockIdx.x * blockDim.x;
  const int r = row0 + threadIdx.x;           // solver row
  const bool active = r < a.N;
  const int node = active ? a.perm[r] : 0;
  const int base = a.prow[row0];
  const int rend = a.prow[min(row0 + (int)blockDim.x, a.N)];
  for (int k = base + threadIdx.x; k < rend; k += blockDim.x) {
    const int j = a.pcol[k];
    sC[k - base] = j;
    sK[k - base] = (a.mode == 1 && a.pbnd[j]) ? 0.0 : a.pK[k];
  }
  int lo = 0, hi = 0;
  bool ident = false;
  double dinv = 1.0, xi = 0.0;
  if (active) {
    lo = a.prow[r] - base;
    hi = a.prow[r + 1] - base;
    ident = a.mode == 1 && a.pbnd[r];
    dinv = a.dinv[node];
    xi = a.x[node];
  }
  __syncthreads();
  auto apply = [&](const double *v) -> double {
    if (ident) return __ldcg(v + r);
    double s = 0.0;
    int k = lo;
    for (; k + 4 <= hi; k += 4) {
      const double v0 = __ldcg(v + sC[k]), v1 = __ldcg(v + sC[k + 1]), v2 = __ldcg(v + sC[k + 2]),
                   v3 = __ldcg(v + sC[k + 3]);
      s += sK[k] * v0; s += sK[k + 1] * v1; s += sK[k + 2] * v2; s += sK[k + 3] * v3;
    }
    for (; k < hi; ++k) s += sK[k] * __ldcg(v + sC[k]);
    return s;
  };
  unsigned epoch = 0;
  // u = M^-1 r: Jacobi, plus (mode 0) the aggregate correction P Ainv P^T r.
  // Every block restricts its own kCGThreads/kAgg aggregates, and after one
  // barrier computes the coarse correction of exactly those aggregates.
  auto precond = [&](double rr, double &uu) -> bool {
    uu = dinv * rr;
    if (!a.coarse) return true;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double s = warp_sum(active ? rr : 0.0);
    if (lane == 0) sagg[wid] = s;
    __syncthreads();
    if (threadIdx.x < kCGThreads / kAgg) {
      const int I = blockIdx.x * (kCGThreads / kAgg) + threadIdx.x;
      if (I < a.nc) a.rc[I] = sagg[2 * threadIdx.x] + sagg[2 * threadIdx.x + 1];
    }
    if (!arrive_wait(a, ++epoch)) return false;
    {
      const int g = threadIdx.x / kAgg, t = threadIdx.x % kAgg;
      const int I = blockIdx.x * (kCGThreads / kAgg) + g;
      double acc = 0.0;
      if (I < a.nc) {
        const double *row = a.ainv + (size_t)I * a.nc;
        for (int J = t; J < a.nc; J += kAgg) acc += row[J] * __ldcg(a.rc + J);
      }
      acc = warp_sum(acc);
      if (lane == 0) sagg[wid] = acc;
      __syncthreads();
      if (threadIdx.x < kCGThreads / kAgg) sec[threadIdx.x] = sagg[2 * threadIdx.x] + sagg[2 * threadIdx.x + 1];
      __syncthreads();
      uu += sec[g];
    }
    return true;
  };
  double mean_b = 0.0;
  const double bi0 = active ? a.b[node] : 0.0;
  if (a.mode == 0) {
    double v[1] = {bi0}, t[1];
    if (!reduce_all<1>(a, ++epoch, v, smem, t)) return;
    mean_b = t[0] / a.N;
  }
  const double bi = active ? bi0 - mean_b : 0.0;
  // ---- projection of b onto the stored right-hand sides ----
  const int count = B.ring[0], head = B.ring[1];
  double proj[kBasis + 1], bdot[kBasis + 1];
#pragma unroll
  for (int j = 0; j <= kBasis; ++j) proj[j] = 0.0;
  if (active) {
#pragma unroll
    for (int j = 0; j < kBasis; ++j) if (j < count) proj[j] = bi * __ldcg(B.b + (size_t)j * a.N + r);
    proj[kBasis] = bi * bi;
  }
  if (!reduce_all<kBasis + 1>(a, ++epoch, proj, smem, bdot)) return;
  const double tol = fmax(a.rtol * sqrt(bdot[kBasis]), a.atol);
  if (count > 0) {
    if (threadIdx.x < 32) small_solve_warp(count, B.gram, bdot, sc, smem);   // reduce scratch is free here
    __syncthreads();
    if (active) {
      double g = 0.0;
      double t[kBasis];   // every load in flight before the sum (same order as a plain loop)
#pragma unroll
      for (int j = 0; j < kBasis; ++j) t[j] = j < count ? __ldcg(B.x + (size_t)j * a.N + r) : 0.0;
#pragma unroll
      for (int j = 0; j < kBasis; ++j) if (j < count) g += sc[j] * t[j];
      xi = ident ? bi : g;   // identity (Dirichlet boundary) rows are exact
    }
  }
  if (active) a.xperm[r] = xi;
  if (!arrive_wait(a, ++epoch)) return;   // publish the initial iterate
  double ri = 0.0, ui = 0.0, pi = 0.0, si = 0.0, wi = 0.0;
  if (active) ri = bi - apply(a.xperm);
  if (!precond(ri, ui)) return;
  if (active) a.z[r] = ui;
  if (!arrive_wait(a, ++epoch)) return;   // publish u
  double gamma = 0.0, alpha = 0.0;
  int it = 0;
  bool failed = false;
  for (;;) {
    double v[3] = {0.0, 0.0, 0.0}, t[3];
    if (active) {
      wi = apply(a.z);
      v[0] = ri * ui; v[1] = wi * ui; v[2] = ri * ri;
    }
    if (!reduce_all<3>(a, ++epoch, v, smem, t)) return;
    // scalar recurrences once per block (FP64 is scarce), broadcast in smem
    if (threadIdx.x == 0) {
      int state = 0;  // 0 continue, 1 converged, 2 failed
      if (!(t[2] == t[2]) || isinf(t[2])) state = 2;
      else if (sqrt(t[2]) <= tol) state = 1;
      else if (it >= a.maxits) state = 2;
      double beta = 0.0, al = alpha;
      if (state == 0) {
        if (it == 0) al = t[0] / t[1];
        else { beta = t[0] / gamma; al = t[0] / (t[1] - beta * t[0] / alpha); }
      }
      sc[0] = al; sc[1] = beta; sc[2] = t[0]; sc[3] = (double)state;
    }
    __syncthreads();
    const int state = (int)sc[3];
    const double beta = sc[1];
    alpha = sc[0];
    gamma = sc[2];
    __syncthreads();
    if (state != 0) { failed = state == 2; break; }
    if (active) {
      pi = ui + beta * pi;
      si = wi + beta * si;
      xi += alpha * pi;
      ri -= alpha * si;
    }
    if (!precond(ri, ui)) return;
    if (active) a.z[r] = ui;
    ++it;
    if (!arrive_wait(a, ++epoch)) return;   // publish the new u
  }
  if (a.mode == 0) {
    double v[1] = {active ? xi : 0.0}, t[1];
    if (!reduce_all<1>(a, ++epoch, v, smem, t)) return;
    xi -= t[0] / a.N;
  }
  if (active) {
    a.x[node] = xi;
    B.b[(size_t)head * a.N + r] = bi;   // remember this solve for the next guess
    B.x[(size_t)head * a.N + r] = xi;
  }
  if (r == 0) {
    a.iters[a.mode] = it;
    a.iters[2 + a.mode] += it;
    if (failed) atomicOr(a.err, ERR_CG_MAXITS);
    // Gram matrix row/column of the slot being replaced: its new vector is b
    const int ncount = count < kBasis ? count + 1 : kBasis;
    for (int j = 0; j < ncount; ++j) {
      const double g = (j == head) ? bdot[kBasis] : bdot[j];
      B.gram[head * kBasis + j] = g;
      B.gram[j * kBasis + head] = g;
    }
    B.ring[0] = ncount;
    B.ring[1] = (head + 1) % kBasis;
  }
}

// Ensemble form of k_cg3: the same persistent single-reduction CG for nm <= MB
// right-hand sides at once (member m's vectors at offset m * N).  A row's
// operator entries are read once for all members; every member has its own
// scalars, stopping test and projection basis (member m's at offset
// m * kBasis * N, gram m * kBasis^2, ring 2m), and is frozen once converged;
// the loop ends when all members have stopped.  Member m's scalar work runs
// on lane 0 of warp m, so the members' FP64 divisions proceed in parallel.
template <int MB>
__global__ void __launch_bounds__(kCGThreads, 1) k_cgm(CGArgs a, int nnz_cap, int nm, CGBasis B) {
  static_assert(MB * 32 <= kCGThreads, "one warp per member for the scalar work");
  constexpr int P = kBasis + 1;
  extern __shared__ double dyn[];
  __shared__ double smem[kCGThreads / 32 * RedShape<P * MB>::W];   // block_reduce_out scratch
  __shared__ double sres[P * MB];                     // totals of the last reduction
  __shared__ double sbdot[P * MB];                    // projection dots (Gram update at the end)
  __shared__ double s_al[MB], s_be[MB], s_ga[MB], s_tol[MB];
  __shared__ int s_st[MB];
  __shared__ int s_cnt[MB], s_head[MB];               // ring read once: block 0 rewrites it at the end
  __shared__ double scoef[MB * kBasis];
  __shared__ double sbi[MB][kCGThreads];              // (centred) right-hand sides of this block's rows
  __shared__ double sagg[MB][2 * (kCGThreads / kAgg)], sec[MB][kCGThreads / kAgg];
  double *sK = dyn;
  int *sC = reinterpret_cast<int *>(sK + nnz_cap);
  const int N = a.N;
  const int tid = threadIdx.x;
  const int row0 = blockIdx.x * blockDim.x;
  const int r = row0 + tid;
  const bool active = r < N;
  const int node = active ? a.perm[r] : 0;
  const int base = a.prow[row0];
  const int rend = a.prow[min(row0 + (int)blockDim.x, N)];
  for (int k = base + tid; k < rend; k += blockDim.x) {
    const int j = a.pcol[k];
    sC[k - base] = j;
    sK[k - base] = (a.mode == 1 && a.pbnd[j]) ? 0.0 : a.pK[k];
  }
  int lo = 0, hi = 0;
  bool ident = false;
  double dinv = 1.0;
  double xi[MB], ri[MB], ui[MB], pi[MB], si[MB], wi[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    xi[m] = ri[m] = ui[m] = pi[m] = si[m] = wi[m] = 0.0;
    sbi[m][tid] = (active && m < nm) ? a.b[(size_t)m * N + node] : 0.0;
  }
  if (active) {
    lo = a.prow[r] - base;
    hi = a.prow[r + 1] - base;
    ident = a.mode == 1 && a.pbnd[r];
    dinv = a.dinv[node];
#pragma unroll
    for (int m = 0; m < MB; ++m) if (m < nm) xi[m] = a.x[(size_t)m * N + node];
  }
  if (tid < MB) {
    s_cnt[tid] = tid < nm ? B.ring[2 * tid] : 0;
    s_head[tid] = tid < nm ? B.ring[2 * tid + 1] : 0;
  }
  __syncthreads();
  // s[m] = (A v_m)_r for every member; published vectors are member-minor
  // (v[row * MB + m]) so that one neighbour's members share cache lines
  auto apply = [&](const double *v, double (&s)[MB]) {
#pragma unroll
    for (int m = 0; m < MB; ++m) s[m] = 0.0;
    if (ident) {
      const double2 *vr = reinterpret_cast<const double2 *>(v + (size_t)r * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) { const double2 t = __ldcg(vr + q); s[2 * q] = t.x; s[2 * q + 1] = t.y; }
      return;
    }
    int k = lo;
    for (; k + 2 <= hi; k += 2) {   // two neighbours' loads in flight
      const double kv0 = sK[k], kv1 = sK[k + 1];
      const double2 *vc0 = reinterpret_cast<const double2 *>(v + (size_t)sC[k] * MB);
      const double2 *vc1 = reinterpret_cast<const double2 *>(v + (size_t)sC[k + 1] * MB);
      double2 t0[MB / 2], t1[MB / 2];
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) { t0[q] = __ldcg(vc0 + q); t1[q] = __ldcg(vc1 + q); }
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        s[2 * q] += kv0 * t0[q].x;
        s[2 * q + 1] += kv0 * t0[q].y;
        s[2 * q] += kv1 * t1[q].x;
        s[2 * q + 1] += kv1 * t1[q].y;
      }
    }
    for (; k < hi; ++k) {
      const double kv = sK[k];
      const double2 *vc = reinterpret_cast<const double2 *>(v + (size_t)sC[k] * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        const double2 t = __ldcg(vc + q);
        s[2 * q] += kv * t.x;
        s[2 * q + 1] += kv * t.y;
      }
    }
  };
  unsigned epoch = 0;
  auto precond = [&](const double (&rr)[MB], double (&uu)[MB]) -> bool {
#pragma unroll
    for (int m = 0; m < MB; ++m) uu[m] = dinv * rr[m];
    if (!a.coarse) return true;
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const double s = warp_sum(active ? rr[m] : 0.0);
      if (lane == 0) sagg[m][wid] = s;
    }
    __syncthreads();
    if (tid < kCGThreads / kAgg) {
      const int I = blockIdx.x * (kCGThreads / kAgg) + tid;
      if (I < a.nc)
        for (int m = 0; m < MB; ++m) a.rc[(size_t)I * MB + m] = sagg[m][2 * tid] + sagg[m][2 * tid + 1];
    }
    if (!arrive_wait(a, ++epoch)) return false;
    const int g = tid / kAgg, t = tid % kAgg;
    const int I = blockIdx.x * (kCGThreads / kAgg) + g;
    double acc[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) acc[m] = 0.0;
    if (I < a.nc) {
      const double *row = a.ainv + (size_t)I * a.nc;
#pragma unroll 2
      for (int J = t; J < a.nc; J += kAgg) {
        const double w = row[J];
        const double2 *rcJ = reinterpret_cast<const double2 *>(a.rc + (size_t)J * MB);
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) {
          const double2 t = __ldcg(rcJ + q);
          acc[2 * q] += w * t.x;
          acc[2 * q + 1] += w * t.y;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const double s = warp_sum(acc[m]);
      if (lane == 0) sagg[m][wid] = s;
    }
    __syncthreads();
    if (tid < kCGThreads / kAgg)
      for (int m = 0; m < nm; ++m) sec[m][tid] = sagg[m][2 * tid] + sagg[m][2 * tid + 1];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < MB; ++m) uu[m] += sec[m][g];
    return true;
  };
  // centre b (Neumann)
  if (a.mode == 0) {
    double v[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) v[m] = sbi[m][tid];
    if (!reduce_all_to<MB>(a, ++epoch, v, smem, sres)) return;
#pragma unroll
    for (int m = 0; m < MB; ++m) if (active) sbi[m][tid] -= sres[m] / N;
  }
  // projection of each member's b onto its stored right-hand sides (+ b.b)
  {
    double proj[P * MB];
#pragma unroll
    for (int q = 0; q < P * MB; ++q) proj[q] = 0.0;
    if (active) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        if (m >= nm) break;
        const int cnt = s_cnt[m];
        const double bm = sbi[m][tid];
        const double *bb = B.b + (size_t)m * kBasis * N;
#pragma unroll
        for (int j = 0; j < kBasis; ++j) if (j < cnt) proj[P * m + j] = bm * bb[(size_t)j * N + r];
        proj[P * m + kBasis] = bm * bm;
      }
    }
    if (!reduce_all_to<P * MB>(a, ++epoch, proj, smem, sbdot)) return;
  }
  if (tid < MB) s_tol[tid] = fmax(a.rtol * sqrt(sbdot[P * tid + kBasis]), a.atol);
  {
    const int m = tid >> 5;
    if (m < nm && s_cnt[m] > 0)   // warp m: member m's coefficients
      small_solve_warp(s_cnt[m], B.gram + m * kBasis * kBasis, sbdot + P * m, scoef + m * kBasis, smem + m * kBasis);
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      if (m >= nm) break;
      const int cnt = s_cnt[m];
      if (cnt == 0) continue;
      const double *bx = B.x + (size_t)m * kBasis * N;
      double g = 0.0;
      double t[kBasis];   // every load in flight before the sum (same order as a plain loop)
#pragma unroll
      for (int j = 0; j < kBasis; ++j) t[j] = j < cnt ? __ldcg(bx + (size_t)j * N + r) : 0.0;
#pragma unroll
      for (int j = 0; j < kBasis; ++j) if (j < cnt) g += scoef[m * kBasis + j] * t[j];
      xi[m] = ident ? sbi[m][tid] : g;
    }
#pragma unroll
    for (int q = 0; q < MB / 2; ++q)
      reinterpret_cast<double2 *>(a.xperm + (size_t)r * MB)[q] = make_double2(xi[2 * q], xi[2 * q + 1]);
  }
  if (!arrive_wait(a, ++epoch)) return;
  {
    double ax[MB];
    apply(a.xperm, ax);
#pragma unroll
    for (int m = 0; m < MB; ++m) ri[m] = active ? sbi[m][tid] - ax[m] : 0.0;
  }
  if (!precond(ri, ui)) return;
  if (active)
#pragma unroll
    for (int q = 0; q < MB / 2; ++q)
      reinterpret_cast<double2 *>(a.z + (size_t)r * MB)[q] = make_double2(ui[2 * q], ui[2 * q + 1]);
  if (tid < MB) { s_al[tid] = 0.0; s_ga[tid] = 0.0; s_be[tid] = 0.0; s_st[tid] = tid < nm ? 0 : 1; }
  if (!arrive_wait(a, ++epoch)) return;
  int it = 0;
  for (;;) {
    {
      double v[3 * MB];
      apply(a.z, wi);
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        v[3 * m] = active ? ri[m] * ui[m] : 0.0;
        v[3 * m + 1] = active ? wi[m] * ui[m] : 0.0;
        v[3 * m + 2] = active ? ri[m] * ri[m] : 0.0;
      }
      if (!reduce_all_to<3 * MB>(a, ++epoch, v, smem, sres)) return;
    }
    {
      const int m = tid >> 5;   // lane 0 of warp m: member m's scalars
      if ((tid & 31) == 0 && m < MB) {
        int st = s_st[m];
        double be = 0.0, al = s_al[m];
        const double t0 = sres[3 * m], t1 = sres[3 * m + 1], t2 = sres[3 * m + 2];
        if (st == 0) {
          if (!(t2 == t2) || isinf(t2)) st = 2;
          else if (sqrt(t2) <= s_tol[m]) st = 1;
          else if (it >= a.maxits) st = 2;
        }
        if (st == 0) {
          if (it == 0) al = t0 / t1;
          else { be = t0 / s_ga[m]; al = t0 / (t1 - be * t0 / s_al[m]); }
          s_ga[m] = t0;
        }
        s_al[m] = al; s_be[m] = be; s_st[m] = st;
      }
    }
    __syncthreads();
    int running = 0;
#pragma unroll
    for (int m = 0; m < MB; ++m) running += s_st[m] == 0;
    if (running == 0) break;
    if (active) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        if (s_st[m] != 0) continue;
        const double al = s_al[m], be = s_be[m];
        pi[m] = ui[m] + be * pi[m];
        si[m] = wi[m] + be * si[m];
        xi[m] += al * pi[m];
        ri[m] -= al * si[m];
      }
    }
    if (!precond(ri, ui)) return;
    if (active)
#pragma unroll
      for (int q = 0; q < MB / 2; ++q)
        reinterpret_cast<double2 *>(a.z + (size_t)r * MB)[q] = make_double2(ui[2 * q], ui[2 * q + 1]);
    ++it;
    if (!arrive_wait(a, ++epoch)) return;
  }
  bool failed = false;
#pragma unroll
  for (int m = 0; m < MB; ++m) failed = failed || s_st[m] == 2;
  __syncthreads();
  if (a.mode == 0) {
    double v[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) v[m] = active ? xi[m] : 0.0;
    if (!reduce_all_to<MB>(a, ++epoch, v, smem, sres)) return;
#pragma unroll
    for (int m = 0; m < MB; ++m) xi[m] -= sres[m] / N;
  }
  if (active) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      if (m >= nm) break;
      const int head = s_head[m];
      a.x[(size_t)m * N + node] = xi[m];
      B.b[(size_t)m * kBasis * N + (size_t)head * N + r] = sbi[m][tid];   // this solve joins the basis
      B.x[(size_t)m * kBasis * N + (size_t)head * N + r] = xi[m];
    }
  }
  if (r == 0) {
    a.iters[a.mode] = it;
    a.iters[2 + a.mode] += it;
    if (failed) atomicOr(a.err, ERR_CG_MAXITS);
  }
  // every block read the ring into shared memory at its start; block 0,
  // lane 0 of warp m updates member m's Gram row/column and ring
  {
    const int m = tid >> 5;
    if (blockIdx.x == 0 && (tid & 31) == 0 && m < nm) {
      double *G = B.gram + m * kBasis * kBasis;
      const int cnt = s_cnt[m], head = s_head[m];
      const int ncount = cnt < kBasis ? cnt + 1 : kBasis;
      for (int j = 0; j < ncount; ++j) {
        const double gv = (j == head) ? sbdot[P * m + kBasis] : sbdot[P * m + j];
        G[head * kBasis + j] = gv;
        G[j * kBasis + head] = gv;
      }
      B.ring[2 * m] = ncount;
      B.ring[2 * m + 1] = (head + 1) % kBasis;
    }
  }
}

// Cross-block total of NV FP32 values: block sums in FP32, accumulated over
// the blocks in FP64 (res, shared).
template <int NV>
__device__ __forceinline__ bool reduce_all_f(const CGArgs &a, unsigned epoch, float (&v)[NV], float *smemf,
                                             double *res) {
  double *slot = a.red + (size_t)(epoch & 1) * gridDim.x * kCG2MaxRed;
  block_reduce_out<float, NV>(v, smemf, slot + blockIdx.x, gridDim.x);
  if (!arrive_wait(a, epoch)) return false;
  grid_total<NV>(slot, res);
  return true;
}

// Mixed-precision form of k_cgm (nm <= MB right-hand sides): FP64 projection
// warm start and FP64 true residual r = b - A x; the correction A d = r is
// solved by the single-reduction CG in FP32 (operator, preconditioner and
// vectors FP32; dot products summed in FP32 within a block and in FP64
// across blocks) to a relative tolerance eta; x += d in FP64; repeated until
// the FP64 residual meets the tolerance (at most max_outer corrections).
// GB300's FP32 pipe is ~60x its FP64 pipe: the inner iterations, where all
// the work is, run on it.
template <int MB>
__global__ void __launch_bounds__(kCGThreads, 1) k_cgm_mp(CGArgs a, int nnz_cap, int nm, CGBasis B) {
  static_assert(MB * 32 <= kCGThreads && MB % 2 == 0, "one warp per member; member pairs");
  constexpr int P = kBasis + 1;
  extern __shared__ double dyn[];
  __shared__ double smem[kCGThreads / 32 * RedShape<(P + 1) * MB>::W];
  __shared__ float smemf[kCGThreads / 32 * RedShape<3 * MB>::W];
  __shared__ double sres[(P + 1) * MB];
  __shared__ double s_xsum[MB];   // sum of x per member at the last FP64 residual (Neumann centring)
  __shared__ double sbdot[P * MB];
  __shared__ double s_tol[MB], s_itol2[MB];
  __shared__ float s_al[MB], s_be[MB], s_ga[MB];
  __shared__ int s_st[MB], s_out[MB];
  __shared__ int s_cnt[MB], s_head[MB];
  __shared__ double scoef[MB * kBasis];
  __shared__ double sbi[MB][kCGThreads];
  __shared__ float sagg[MB][2 * (kCGThreads / kAgg)], sec[MB][kCGThreads / kAgg];
  double *sK = dyn;
  int *sC = reinterpret_cast<int *>(sK + nnz_cap);
  float *sK32 = reinterpret_cast<float *>(sC + nnz_cap);
  const int N = a.N;
  const int tid = threadIdx.x;
  const int row0 = blockIdx.x * blockDim.x;
  const int r = row0 + tid;
  const bool active = r < N;
  const int node = active ? a.perm[r] : 0;
  const int base = a.prow[row0];
  const int rend = a.prow[min(row0 + (int)blockDim.x, N)];
  {   // the block's rows in their shared-memory order (made at setup): in each row
      // the columns inside the block's row range first, applied from the block's
      // own u while the barrier that publishes u completes; independent loads only
    const double *mK = a.mode == 1 ? a.mK1 : a.mK0;
    const float *mK32 = a.mode == 1 ? a.mK32_1 : a.mK32_0;
#pragma unroll 4
    for (int k = base + tid; k < rend; k += blockDim.x) {
      sC[k - base] = __ldg(a.mcol + k);
      sK[k - base] = __ldg(mK + k);
      sK32[k - base] = __ldg(mK32 + k);
    }
  }
  int lo = 0, hi = 0, mid = 0;
  bool ident = false;
  double dinv = 1.0;
  double xi[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    xi[m] = 0.0;
    sbi[m][tid] = (active && m < nm) ? a.b[(size_t)m * N + node] : 0.0;
  }
  if (active) {
    lo = a.prow[r] - base;
    hi = a.prow[r + 1] - base;
    mid = lo + a.mmid[r];
    ident = a.mode == 1 && a.pbnd[r];
    dinv = a.dinv[node];
#pragma unroll
    for (int m = 0; m < MB; ++m) if (m < nm) xi[m] = a.x[(size_t)m * N + node];
  }
  const float dinv32 = (float)dinv;
  float *suS = sK32 + nnz_cap;                        // this block's u, kCGThreads x MB (local SpMV)
  float *rcS = suS + (size_t)kCGThreads * MB;         // coarse residual R r of every aggregate (nc x MB)
  float *RsS = rcS + (size_t)a.nc * MB;               // R s of every aggregate (nc x MB)
  float *ainvS = RsS + (size_t)a.nc * MB;             // this block's rows of the coarse inverse
  if (a.coarse)
    for (int e = tid; e < (kCGThreads / kAgg) * a.nc; e += kCGThreads) {
      const int I = blockIdx.x * (kCGThreads / kAgg) + e / a.nc;
      ainvS[e] = I < a.nc ? a.ainv32[(size_t)I * a.nc + e % a.nc] : 0.f;
    }

  if (tid < MB) {
    s_cnt[tid] = tid < nm ? B.ring[2 * tid] : 0;
    s_head[tid] = tid < nm ? B.ring[2 * tid + 1] : 0;
  }
  __syncthreads();
  // FP64 operator on the published member-minor FP64 vector
  auto apply64 = [&](const double *v, double (&s)[MB]) {
#pragma unroll
    for (int m = 0; m < MB; ++m) s[m] = 0.0;
    if (ident) {
      const double2 *vr = reinterpret_cast<const double2 *>(v + (size_t)r * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) { const double2 t = __ldcg(vr + q); s[2 * q] = t.x; s[2 * q + 1] = t.y; }
      return;
    }
    int k = lo;
    for (; k + 2 <= hi; k += 2) {   // two neighbours' loads in flight
      const double kv0 = sK[k], kv1 = sK[k + 1];
      const double2 *vc0 = reinterpret_cast<const double2 *>(v + (size_t)sC[k] * MB);
      const double2 *vc1 = reinterpret_cast<const double2 *>(v + (size_t)sC[k + 1] * MB);
      double2 t0[MB / 2], t1[MB / 2];
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) { t0[q] = __ldcg(vc0 + q); t1[q] = __ldcg(vc1 + q); }
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        s[2 * q] += kv0 * t0[q].x;
        s[2 * q + 1] += kv0 * t0[q].y;
        s[2 * q] += kv1 * t1[q].x;
        s[2 * q + 1] += kv1 * t1[q].y;
      }
    }
    for (; k < hi; ++k) {
      const double kv = sK[k];
      const double2 *vc = reinterpret_cast<const double2 *>(v + (size_t)sC[k] * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        const double2 t = __ldcg(vc + q);
        s[2 * q] += kv * t.x;
        s[2 * q + 1] += kv * t.y;
      }
    }
  };
  // FP32 operator, in two parts around the barrier that publishes u: the
  // columns inside this block's row range (put first in each row, above)
  // from the block's own u in shared memory, before the wait; the other
  // columns from the published member-minor FP32 vector, after it.
  auto apply32_local = [&](float (&s)[MB]) {
#pragma unroll
    for (int m = 0; m < MB; ++m) s[m] = 0.f;
    if (ident) {
      const float2 *vr = reinterpret_cast<const float2 *>(suS + (size_t)tid * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) { const float2 t = vr[q]; s[2 * q] = t.x; s[2 * q + 1] = t.y; }
      return;
    }
    for (int k = lo; k < mid; ++k) {
      const float kv = sK32[k];
      const float2 *vc = reinterpret_cast<const float2 *>(suS + (size_t)(sC[k] - row0) * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        const float2 t = vc[q];
        s[2 * q] = fmaf(kv, t.x, s[2 * q]);
        s[2 * q + 1] = fmaf(kv, t.y, s[2 * q + 1]);
      }
    }
  };
  auto apply32_halo = [&](const float *v, float (&s)[MB]) {
    if (ident) return;
    int k = mid;
    for (; k + 4 <= hi; k += 4) {   // four neighbours' loads in flight
      float2 t[4][MB / 2];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float2 *vc = reinterpret_cast<const float2 *>(v + (size_t)sC[k + u] * MB);
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) t[u][q] = __ldcg(vc + q);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float kv = sK32[k + u];
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) {
          s[2 * q] = fmaf(kv, t[u][q].x, s[2 * q]);
          s[2 * q + 1] = fmaf(kv, t[u][q].y, s[2 * q + 1]);
        }
      }
    }
    for (; k < hi; ++k) {
      const float kv = sK32[k];
      const float2 *vc = reinterpret_cast<const float2 *>(v + (size_t)sC[k] * MB);
#pragma unroll
      for (int q = 0; q < MB / 2; ++q) {
        const float2 t = __ldcg(vc + q);
        s[2 * q] = fmaf(kv, t.x, s[2 * q]);
        s[2 * q + 1] = fmaf(kv, t.y, s[2 * q + 1]);
      }
    }
  };
  unsigned epoch = 0;
  // Two-level preconditioner u = D^-1 r + P A_c^-1 R r (R: sums over the
  // kAgg-row aggregates; a block's rows form whole aggregates).  Every block
  // keeps the whole coarse residual R r in shared memory (rcS): precond32
  // forms it from r (one barrier) at the start of an inner solve; inside the
  // iteration it follows the recurrence R r -= alpha R s, R s = R w + beta R s,
  // with R w published alongside the dot products, so the coarse step needs
  // no barrier of its own.
  auto coarse_add = [&](float (&uu)[MB]) {
    const int lane = tid & 31, wid = tid >> 5;
    const int g = tid / kAgg, t = tid % kAgg;
    const int I = blockIdx.x * (kCGThreads / kAgg) + g;
    float acc[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) acc[m] = 0.f;
    if (I < a.nc) {
      const float *row = ainvS + (size_t)g * a.nc;
#pragma unroll 4
      for (int J = t; J < a.nc; J += kAgg) {
        const float w = row[J];
        const float2 *rcJ = reinterpret_cast<const float2 *>(rcS + (size_t)J * MB);
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) {
          const float2 tt = rcJ[q];
          acc[2 * q] = fmaf(w, tt.x, acc[2 * q]);
          acc[2 * q + 1] = fmaf(w, tt.y, acc[2 * q + 1]);
        }
      }
    }
    {
      constexpr int SH = MB == 8 ? 2 : (MB == 4 ? 3 : 4);
      const float tot = warp_transpose_sum<float, MB>(acc);   // lane L: member L >> SH
      if ((lane & ((1 << SH) - 1)) == 0) sagg[lane >> SH][wid] = tot;
    }
    __syncthreads();
    if (tid < (kCGThreads / kAgg) * MB) {
      const int gg = tid / MB, m = tid % MB;
      sec[m][gg] = sagg[m][2 * gg] + sagg[m][2 * gg + 1];
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < MB; ++m) uu[m] += sec[m][g];
  };
  // block sums of v over this block's aggregates, written to out[I * MB + m]
  auto aggregate_sums = [&](const float (&v)[MB], float *out) {
    const int lane = tid & 31, wid = tid >> 5;
    float w[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) w[m] = active ? v[m] : 0.f;
    constexpr int SH = MB == 8 ? 2 : (MB == 4 ? 3 : 4);
    const float tot = warp_transpose_sum<float, MB>(w);
    if ((lane & ((1 << SH) - 1)) == 0) sagg[lane >> SH][wid] = tot;
    __syncthreads();
    if (tid < (kCGThreads / kAgg) * MB) {
      const int gg = tid / MB, m = tid % MB;
      const int I = blockIdx.x * (kCGThreads / kAgg) + gg;
      if (I < a.nc) out[(size_t)I * MB + m] = sagg[m][2 * gg] + sagg[m][2 * gg + 1];
    }
  };
  // Local part of the preconditioner: u = D^-1 r, then local_sweeps - 1
  // damped Jacobi sweeps u += (2/3) D^-1 (r - A_loc u) with A_loc the
  // block's own rows and columns (its subdomain, the other blocks' values
  // taken as zero): a polynomial in D^-1 A_loc times D^-1, so the
  // preconditioner stays symmetric positive definite (additive Schwarz with
  // an inexact subdomain solve; the coarse level is added to it).  Uses suS
  // as scratch; with one sweep it is the Jacobi step alone.
  auto local_smooth = [&](const float (&rr)[MB], float (&uu)[MB]) {
#pragma unroll
    for (int m = 0; m < MB; ++m) uu[m] = dinv32 * rr[m];
    for (int sw = 1; sw < a.local_sweeps; ++sw) {
#pragma unroll
      for (int q = 0; q < MB / 2; ++q)
        reinterpret_cast<float2 *>(suS + (size_t)tid * MB)[q] =
            active ? make_float2(uu[2 * q], uu[2 * q + 1]) : make_float2(0.f, 0.f);
      __syncthreads();
      float au[MB];
      apply32_local(au);
      __syncthreads();
#pragma unroll
      for (int m = 0; m < MB; ++m) uu[m] = fmaf((2.f / 3.f) * dinv32, rr[m] - au[m], uu[m]);
    }
  };
  auto precond32 = [&](const float (&rr)[MB], float (&uu)[MB]) -> bool {
    local_smooth(rr, uu);
    if (!a.coarse) return true;
    aggregate_sums(rr, a.rc32);
    if (!arrive_wait(a, ++epoch)) return false;
    for (int e = tid; e < a.nc * MB; e += kCGThreads) {
      rcS[e] = __ldcg(a.rc32 + e);
      RsS[e] = 0.f;
    }
    __syncthreads();
    coarse_add(uu);
    return true;
  };
  // ---- projection warm start (FP64).  For the Neumann problem the sum of b
  // rides on the same reduction: the stored right-hand sides are centred, so
  // (b - mean) . b_j = b . b_j to rounding and |b - mean|^2 = b . b - N mean^2.
  {
    constexpr int PP = P + 1;
    double proj[PP * MB];
#pragma unroll
    for (int q = 0; q < PP * MB; ++q) proj[q] = 0.0;
    if (active) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        if (m >= nm) break;
        const int cnt = s_cnt[m];
        const double bm = sbi[m][tid];
        const double *bb = B.b + (size_t)m * kBasis * N;
#pragma unroll
        for (int j = 0; j < kBasis; ++j) if (j < cnt) proj[PP * m + j] = bm * bb[(size_t)j * N + r];
        proj[PP * m + kBasis] = bm * bm;
        proj[PP * m + kBasis + 1] = bm;
      }
    }
    if (!reduce_all_to<PP * MB>(a, ++epoch, proj, smem, sres)) return;
    for (int q = tid; q < P * MB; q += kCGThreads) {
      const int m = q / P, j = q - m * P;
      const double mean = a.mode == 0 ? sres[PP * m + kBasis + 1] / N : 0.0;
      sbdot[q] = j < kBasis ? sres[PP * m + j] : sres[PP * m + kBasis] - N * mean * mean;
    }
    if (a.mode == 0)
#pragma unroll
      for (int m = 0; m < MB; ++m) if (active) sbi[m][tid] -= sres[PP * m + kBasis + 1] / N;
    __syncthreads();
  }
  if (tid < MB) s_tol[tid] = fmax(a.rtol * sqrt(sbdot[P * tid + kBasis]), a.atol);
  {
    const int m = tid >> 5, lane = tid & 31;
    if (m < nm && s_cnt[m] > 0) {   // warp m: member m's coefficients
      const GramLDL *f = B.ldl ? B.ldl + m : nullptr;
      if (f && __ldcg(&f->n) == s_cnt[m]) {   // factored after this basis's last solve: substitute only
        double L[kBasis];
        const double rd = lane < kBasis ? __ldcg(f->rd + lane) : 0.0;
#pragma unroll
        for (int j = 0; j < kBasis; ++j) L[j] = lane < kBasis ? __ldcg(f->L + lane * kBasis + j) : 0.0;
        small_subst_warp(s_cnt[m], L, rd, __ldcg(&f->on), sbdot + P * m, scoef + m * kBasis);
      } else {
        small_solve_warp(s_cnt[m], B.gram + m * kBasis * kBasis, sbdot + P * m, scoef + m * kBasis,
                         smem + m * kBasis);
      }
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      if (m >= nm) break;
      const int cnt = s_cnt[m];
      if (cnt == 0) continue;
      const double *bx = B.x + (size_t)m * kBasis * N;
      double g = 0.0;
      double t[kBasis];   // every load in flight before the sum (same order as a plain loop)
#pragma unroll
      for (int j = 0; j < kBasis; ++j) t[j] = j < cnt ? __ldcg(bx + (size_t)j * N + r) : 0.0;
#pragma unroll
      for (int j = 0; j < kBasis; ++j) if (j < cnt) g += scoef[m * kBasis + j] * t[j];
      xi[m] = ident ? sbi[m][tid] : g;
    }
  }
  int it = 0;
  bool failed = false;
  // ---- FP64 refinement loop ----
  for (int outer = 0;; ++outer) {
    if (active)
#pragma unroll
      for (int q = 0; q < MB / 2; ++q)
        reinterpret_cast<double2 *>(a.xperm + (size_t)r * MB)[q] = make_double2(xi[2 * q], xi[2 * q + 1]);
    if (!arrive_wait(a, ++epoch)) return;
    double r64[MB];
    {
      double ax[MB];
      apply64(a.xperm, ax);
      double v[2 * MB];   // |r|^2, and sum of x for the Neumann centring at the end
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        r64[m] = active ? sbi[m][tid] - ax[m] : 0.0;
        v[m] = r64[m] * r64[m];
        v[MB + m] = (a.mode == 0 && active) ? xi[m] : 0.0;
      }
      if (!reduce_all_to<2 * MB>(a, ++epoch, v, smem, sres)) return;
    }
    if (tid < MB) {
      const double rn = sres[tid];
      s_xsum[tid] = sres[MB + tid];
      int st = (tid < nm && !(sqrt(rn) <= s_tol[tid])) ? 0 : 1;
      if (!(rn == rn)) st = 2;
      s_out[tid] = st;
      // inner target: the reduction still needed (with margin), but at least eta
      const double itol = fmax(0.5 * s_tol[tid], (double)a.eta * sqrt(rn));
      s_itol2[tid] = itol * itol;
    }
    __syncthreads();
    int open = 0;
#pragma unroll
    for (int m = 0; m < MB; ++m) { open += s_out[m] == 0; failed = failed || s_out[m] == 2; }
    if (open == 0 || failed) break;
    if (outer >= a.max_outer) { failed = true; break; }
    // ---- inner FP32 CG on A d = r for the open members ----
    float ri[MB], ui[MB], pi[MB], si[MB], wi[MB], di[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      ri[m] = (s_out[m] == 0) ? (float)r64[m] : 0.f;
      ui[m] = pi[m] = si[m] = wi[m] = di[m] = 0.f;
    }
    if (!precond32(ri, ui)) return;
    // publish u (global for the other blocks, shared for this block's rows)
    auto publish = [&]() {
      if (active)
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) {
          const float2 t = make_float2(ui[2 * q], ui[2 * q + 1]);
          reinterpret_cast<float2 *>(a.z32 + (size_t)r * MB)[q] = t;
          reinterpret_cast<float2 *>(suS + (size_t)tid * MB)[q] = t;
        }
      else
#pragma unroll
        for (int q = 0; q < MB / 2; ++q) reinterpret_cast<float2 *>(suS + (size_t)tid * MB)[q] = make_float2(0.f, 0.f);
    };
    publish();
    if (tid < MB) { s_al[tid] = 0.f; s_ga[tid] = 0.f; s_be[tid] = 0.f; s_st[tid] = s_out[tid] == 0 ? 0 : 1; }
    arrive(a);
    apply32_local(wi);
    if (!wait_epoch(a, ++epoch)) return;
    int iit = 0;
    for (;;) {
      {
        float v[3 * MB];
        apply32_halo(a.z32, wi);
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          v[3 * m] = active ? ri[m] * ui[m] : 0.f;
          v[3 * m + 1] = active ? wi[m] * ui[m] : 0.f;
          v[3 * m + 2] = active ? ri[m] * ri[m] : 0.f;
        }
        if (a.coarse) aggregate_sums(wi, a.rw32);   // R w rides on the reduction's barrier
        if (!reduce_all_f<3 * MB>(a, ++epoch, v, smemf, sres)) return;
      }
      // this thread's share of every aggregate's R w, loaded while the scalars are formed
      float4 rwq[kRwPer];
      if (a.coarse)
#pragma unroll
        for (int q = 0; q < kRwPer; ++q) {
          const int e4 = tid + q * kCGThreads;
          rwq[q] = e4 * 4 < a.nc * MB ? __ldcg(reinterpret_cast<const float4 *>(a.rw32) + e4)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      {
        const int m = tid >> 5;   // lane 0 of warp m: member m's scalars (FP32, like the vectors)
        if ((tid & 31) == 0 && m < MB) {
          int st = s_st[m];
          float be = 0.f, al = s_al[m];
          const double t0 = sres[3 * m], t1 = sres[3 * m + 1], t2 = sres[3 * m + 2];
          const float f0 = (float)t0, f1 = (float)t1;
          if (st == 0) {
            if (!(t2 == t2) || isinf(t2)) st = 2;
            else if (t2 <= s_itol2[m] || !(f1 > 0.f)) st = 1;
            else if (it + iit >= a.maxits) st = 2;
          }
          if (st == 0) {
            if (iit == 0) al = f0 / f1;
            else {
              be = f0 / s_ga[m];
              const float den = f1 - be * f0 / s_al[m];
              if (den > 0.f) al = f0 / den;
              else st = 1;   // lost positivity in FP32: end this inner solve, the FP64 loop continues
            }
            s_ga[m] = f0;
          }
          s_al[m] = al; s_be[m] = be; s_st[m] = st;
        }
      }
      __syncthreads();
      int running = 0;
#pragma unroll
      for (int m = 0; m < MB; ++m) { running += s_st[m] == 0; failed = failed || s_st[m] == 2; }
      if (running == 0) break;
      if (a.coarse) {   // R s = R w + beta R s, R r -= alpha R s (every aggregate, every block)
#pragma unroll
        for (int q = 0; q < kRwPer; ++q) {
          const int e4 = tid + q * kCGThreads;
          if (e4 * 4 >= a.nc * MB) continue;
          const float rw[4] = {rwq[q].x, rwq[q].y, rwq[q].z, rwq[q].w};
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int e = 4 * e4 + c, m = e & (MB - 1);
            if (e >= a.nc * MB || s_st[m] != 0) continue;
            const float rs = fmaf(s_be[m], RsS[e], rw[c]);
            RsS[e] = rs;
            rcS[e] = fmaf(-s_al[m], rs, rcS[e]);
          }
        }
        __syncthreads();
      }
      if (active) {
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          if (s_st[m] != 0) continue;
          const float al = s_al[m], be = s_be[m];
          pi[m] = fmaf(be, pi[m], ui[m]);
          si[m] = fmaf(be, si[m], wi[m]);
          di[m] = fmaf(al, pi[m], di[m]);
          ri[m] = fmaf(-al, si[m], ri[m]);
        }
      }
      local_smooth(ri, ui);
      if (a.coarse) coarse_add(ui);
      publish();
      ++iit;
      arrive(a);
      apply32_local(wi);
      if (!wait_epoch(a, ++epoch)) return;
    }
    it += iit;
    if (failed) break;
#pragma unroll
    for (int m = 0; m < MB; ++m) if (s_out[m] == 0) xi[m] += (double)di[m];
  }
  __syncthreads();
  if (a.mode == 0)   // x is unchanged since the last residual reduction summed it
#pragma unroll
    for (int m = 0; m < MB; ++m) xi[m] -= s_xsum[m] / N;
  if (active) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      if (m >= nm) break;
      const int head = s_head[m];
      a.x[(size_t)m * N + node] = xi[m];
      B.b[(size_t)m * kBasis * N + (size_t)head * N + r] = sbi[m][tid];
      B.x[(size_t)m * kBasis * N + (size_t)head * N + r] = xi[m];
    }
  }
  if (r == 0) {
    a.iters[a.mode] = it;
    a.iters[2 + a.mode] += it;
    if (failed) atomicOr(a.err, ERR_CG_MAXITS);
  }
  {
    const int m = tid >> 5;
    if (blockIdx.x == 0 && (tid & 31) == 0 && m < nm) {
      double *G = B.gram + m * kBasis * kBasis;
      const int cnt = s_cnt[m], head = s_head[m];
      const int ncount = cnt < kBasis ? cnt + 1 : kBasis;
      for (int j = 0; j < ncount; ++j) {
        const double gv = (j == head) ? sbdot[P * m + kBasis] : sbdot[P * m + j];
        G[head * kBasis + j] = gv;
        G[j * kBasis + head] = gv;
      }
      B.ring[2 * m] = ncount;
      B.ring[2 * m + 1] = (head + 1) % kBasis;
    }
  }
}

__global__ void k_dinv(int N, const int32_t *__restrict__ diag_pos, const double *__restrict__ K,
                       const int32_t *__restrict__ b_of_node, double *__restrict__ dn, double *__restrict__ dd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double inv = 1.0 / K[diag_pos[i]];
  dn[i] = inv;
  dd[i] = b_of_node[i] >= 0 ? 1.0 : inv;
}

// rho = -(Ms * sum_k (D_x m_x + D_y m_y + D_z m_z))
__global__ void k_div(int N, int nnz, double Ms, const int32_t *__restrict__ row_ptr,
                      const int32_t *__restrict__ col_idx, const double *__restrict__ D,
                      const double *__restrict__ m, double *__restrict__ rho, int nrep = 1) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)N * nrep) return;
  const int b = (int)(g / N), i = (int)(g - (long long)b * N);
  const double *mb = m + (size_t)b * 3 * N;
  double s = 0.0;
  for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
    const double *mj = mb + 3 * (size_t)col_idx[k];
    s += (D[k] * mj[0] + D[(size_t)nnz + k] * mj[1]) + D[2 * (size_t)nnz + k] * mj[2];
  }
  rho[g] = -(Ms * s);
}

__global__ void k_gather_b(int nb, const int32_t *__restrict__ node_of_b, const double *__restrict__ phi,
                           double *__restrict__ out, int N = 0, int nrep = 1) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nb * nrep) return;
  const int mbr = g / nb, j = g - mbr * nb;
  out[g] = phi[(size_t)mbr * N + node_of_b[j]];
}

// BEM product y = B x over the row-major matrix (row stride ld, a multiple of
// 8; pad columns zero).  The matrix is streamed as one flat sequence of
// 32-byte units (4 FP64 or 8 FP32 entries); warp w owns the contiguous unit
// range [w*seg, (w+1)*seg), so every warp streams the same number of bytes
// whatever nb is, with no partial last wave.  A warp's range crosses at most
// a few row ends: per row it touches, the lanes' sums are combined by a fixed
// shuffle tree and lane 0 stores one partial, part[w*maxr + (row - first row
// of w)].  k_row_sum adds a row's partials in warp order, so the result is
// deterministic for a given grid.
constexpr int kGemvThreads = 256;
constexpr int kGemvUnroll = 4;

__global__ void __launch_bounds__(kGemvThreads) k_gemv_f64(int nb, int ld, long long seg, int maxr,
                                                            const double *__restrict__ B,
                                                            const double *__restrict__ x, double *__restrict__ part) {
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long Q = ld / 4, total = (long long)nb * Q;
  const long long q0 = w * seg, q1 = min(total, q0 + seg);
  if (q0 >= q1) return;
  const long long rfirst = q0 / Q;
  for (long long r = rfirst; r * Q < q1; ++r) {
    const long long a = max(q0, r * Q), e = min(q1, (r + 1) * Q);
    const double *row = B + r * (long long)ld;
    double acc0 = 0.0, acc1 = 0.0;
    long long q = a + lane;
    for (; q + 32 * (kGemvUnroll - 1) < e; q += 32 * kGemvUnroll) {
      double2 v[kGemvUnroll][2];
#pragma unroll
      for (int u = 0; u < kGemvUnroll; ++u) {
        const double2 *p = reinterpret_cast<const double2 *>(row + 4 * (q - r * Q + 32 * u));
        v[u][0] = __ldcs(p);
        v[u][1] = __ldcs(p + 1);
      }
#pragma unroll
      for (int u = 0; u < kGemvUnroll; ++u) {
        const int c = (int)(4 * (q - r * Q + 32 * u));
        acc0 = fma(v[u][0].x, __ldg(x + min(c, nb - 1)), acc0);
        acc1 = fma(v[u][0].y, __ldg(x + min(c + 1, nb - 1)), acc1);
        acc0 = fma(v[u][1].x, __ldg(x + min(c + 2, nb - 1)), acc0);
        acc1 = fma(v[u][1].y, __ldg(x + min(c + 3, nb - 1)), acc1);
      }
    }
    for (; q < e; q += 32) {
      const double2 *p = reinterpret_cast<const double2 *>(row + 4 * (q - r * Q));
      const double2 v0 = __ldcs(p), v1 = __ldcs(p + 1);
      const int c = (int)(4 * (q - r * Q));
      acc0 = fma(v0.x, __ldg(x + min(c, nb - 1)), acc0);
      acc1 = fma(v0.y, __ldg(x + min(c + 1, nb - 1)), acc1);
      acc0 = fma(v1.x, __ldg(x + min(c + 2, nb - 1)), acc0);
      acc1 = fma(v1.y, __ldg(x + min(c + 3, nb - 1)), acc1);
    }
    const double s = warp_sum(acc0 + acc1);
    if (lane == 0) part[w * maxr + (r - rfirst)] = s;
  }
}

// FP32 matrix, x32 zero-padded to ld: products summed in FP32 per 32-entry
// group of a lane, groups summed in FP64.
__global__ void __launch_bounds__(kGemvThreads) k_gemv_f32(int nb, int ld, long long seg, int maxr,
                                                            const float *__restrict__ B,
                                                            const float *__restrict__ x, double *__restrict__ part,
                                                            const int *__restrict__ gate = nullptr) {
  if (gate && *gate) return;   // anchored product: this chunk refreshes its anchor instead
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long Q = ld / 8, total = (long long)nb * Q;
  const long long q0 = w * seg, q1 = min(total, q0 + seg);
  if (q0 >= q1) return;
  const long long rfirst = q0 / Q;
  for (long long r = rfirst; r * Q < q1; ++r) {
    const long long a = max(q0, r * Q), e = min(q1, (r + 1) * Q);
    const float *row = B + r * (long long)ld;
    double acc = 0.0;
    long long q = a + lane;
    for (; q + 32 * (kGemvUnroll - 1) < e; q += 32 * kGemvUnroll) {
      float4 v[kGemvUnroll][2];
#pragma unroll
      for (int u = 0; u < kGemvUnroll; ++u) {
        const float4 *p = reinterpret_cast<const float4 *>(row + 8 * (q - r * Q + 32 * u));
        v[u][0] = __ldcs(p);
        v[u][1] = __ldcs(p + 1);
      }
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int u = 0; u < kGemvUnroll; ++u) {
        const float4 *px = reinterpret_cast<const float4 *>(x + 8 * (q - r * Q + 32 * u));
        const float4 x0 = __ldg(px), x1 = __ldg(px + 1);
        s0 = fmaf(v[u][0].x, x0.x, s0); s1 = fmaf(v[u][0].y, x0.y, s1);
        s0 = fmaf(v[u][0].z, x0.z, s0); s1 = fmaf(v[u][0].w, x0.w, s1);
        s0 = fmaf(v[u][1].x, x1.x, s0); s1 = fmaf(v[u][1].y, x1.y, s1);
        s0 = fmaf(v[u][1].z, x1.z, s0); s1 = fmaf(v[u][1].w, x1.w, s1);
      }
      acc += (double)(s0 + s1);
    }
    for (; q < e; q += 32) {
      const float4 *p = reinterpret_cast<const float4 *>(row + 8 * (q - r * Q));
      const float4 *px = reinterpret_cast<const float4 *>(x + 8 * (q - r * Q));
      const float4 v0 = __ldcs(p), v1 = __ldcs(p + 1), x0 = __ldg(px), x1 = __ldg(px + 1);
      float s0 = v0.x * x0.x;
      s0 = fmaf(v0.y, x0.y, s0); s0 = fmaf(v0.z, x0.z, s0); s0 = fmaf(v0.w, x0.w, s0);
      s0 = fmaf(v1.x, x1.x, s0); s0 = fmaf(v1.y, x1.y, s0); s0 = fmaf(v1.z, x1.z, s0); s0 = fmaf(v1.w, x1.w, s0);
      acc += (double)s0;
    }
    const double s = warp_sum(acc);
    if (lane == 0) part[w * maxr + (r - rfirst)] = s;
  }
}

// y[r] = sum of the partials of the warps whose unit range meets row r, in
// warp order (Q = units per row).
__global__ void k_row_sum(int nb, long long Q, long long seg, int maxr, long long nwarps,
                          const double *__restrict__ part, double *__restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  const long long w0 = (r * Q) / seg, w1 = min(nwarps - 1, ((r + 1) * Q - 1) / seg);
  double s = 0.0;
  for (long long w = w0; w <= w1; ++w) s += part[w * maxr + (r - (w * seg) / Q)];
  y[r] = s;
}

__global__ void k_to_f32_vec(int n, int ld, const double *__restrict__ a, float *__restrict__ b, int nm = 1) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ld * nm) return;
  const int m = g / ld, i = g - m * ld;
  b[g] = i < n ? (float)a[(size_t)m * n + i] : 0.0f;
}

// Ensemble BEM products Y = B X for nm <= MB members (x member m at m * nb,
// FP32 copies at m * ld, zero-padded): the warp-segment decomposition of
// k_gemv_*, every matrix unit multiplied into all members' accumulators, so
// the matrix is streamed once per nm right-hand sides.  Partials at
// part[(w * maxr + row slot) * MB + m].
template <int MB>
__global__ void __launch_bounds__(kGemvThreads) k_gemm_f64(int nb, int ld, long long seg, int maxr, int nm,
                                                            const double *__restrict__ B,
                                                            const double *__restrict__ x, double *__restrict__ part) {
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long Q = ld / 4, total = (long long)nb * Q;
  const long long q0 = w * seg, q1 = min(total, q0 + seg);
  if (q0 >= q1) return;
  const long long rfirst = q0 / Q;
  for (long long r = rfirst; r * Q < q1; ++r) {
    const long long a = max(q0, r * Q), e = min(q1, (r + 1) * Q);
    const double *row = B + r * (long long)ld;
    double acc[MB];
#pragma unroll
    for (int m = 0; m < MB; ++m) acc[m] = 0.0;
    for (long long q = a + lane; q < e; q += 32) {
      const double2 *p = reinterpret_cast<const double2 *>(row + 4 * (q - r * Q));
      const double2 v0 = __ldcs(p), v1 = __ldcs(p + 1);
      const int c = (int)(4 * (q - r * Q));
      const int c0 = min(c, nb - 1), c1 = min(c + 1, nb - 1), c2 = min(c + 2, nb - 1), c3 = min(c + 3, nb - 1);
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        if (m >= nm) break;
        const double *xm = x + (size_t)m * nb;
        double t = fma(v0.x, __ldg(xm + c0), acc[m]);
        t = fma(v0.y, __ldg(xm + c1), t);
        t = fma(v1.x, __ldg(xm + c2), t);
        acc[m] = fma(v1.y, __ldg(xm + c3), t);
      }
    }
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      if (m >= nm) break;
      const double s = warp_sum(acc[m]);
      if (lane == 0) part[(w * maxr + (r - rfirst)) * MB + m] = s;
    }
  }
}

constexpr int kTileRpw = 4;   // rows per warp step of the FP32 ensemble product


// FP32 ensemble product, x held in registers: block (slab group, row block)
// covers kRegSlab columns with its 8 warps, warp w owning 256 columns and
// lane l the 8 columns at 256 w + 8 l, for which it keeps every member's x
// in registers.  The warp walks the block's rows kTileRpw at a time (one
// 32-byte load per row and lane, no shared-memory x traffic), reduces its
// kTileRpw x MB sums across lanes (FP32: each covers the warp's 256 columns),
// and parks them in shared memory; the 8 warps' sums are added in FP64 once
// at the end.  part[(slab group * nb + row) * MB + m].
constexpr int kRegSlab = 2048, kRegRows = 64;   // 32 KB of shared sums at MB = 8

template <int MB>
__global__ void __launch_bounds__(256, 2) k_gemm_f32r(int nb, int ld, int nm, const float *__restrict__ B,
                                                      const float *__restrict__ x, double *__restrict__ part,
                                                      const int *__restrict__ gate = nullptr) {
  if (gate && *gate) return;   // anchored product: this chunk refreshes its anchor instead
  constexpr int NV = kTileRpw * MB;
  constexpr int SH = NV >= 32 ? 0 : (NV >= 16 ? 1 : (NV >= 8 ? 2 : 3));
  constexpr int STEPS = kRegRows / kTileRpw;
  __shared__ double sred[8][STEPS][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = blockIdx.x * kRegSlab + 256 * warp + 8 * lane;
  const bool on = c < ld;   // ld is a multiple of 8: a lane's unit is all in or all out
  float4 xr[MB][2];
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    const bool ok = on && m < nm;
    const float4 *px = reinterpret_cast<const float4 *>(x + (size_t)m * ld + (ok ? c : 0));
    xr[m][0] = ok ? __ldg(px) : make_float4(0.f, 0.f, 0.f, 0.f);
    xr[m][1] = ok ? __ldg(px + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  const int rbeg = blockIdx.y * kRegRows;
  for (int st = 0; st < STEPS; ++st) {
    const int r0 = rbeg + st * kTileRpw;
    if (r0 >= nb) break;   // uniform across the block
    float4 a[kTileRpw][2];
#pragma unroll
    for (int rr = 0; rr < kTileRpw; ++rr) {
      const float4 *p = reinterpret_cast<const float4 *>(B + (size_t)min(r0 + rr, nb - 1) * ld + (on ? c : 0));
      a[rr][0] = on ? __ldcs(p) : make_float4(0.f, 0.f, 0.f, 0.f);
      a[rr][1] = on ? __ldcs(p + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float acc[NV];
#pragma unroll
    for (int rr = 0; rr < kTileRpw; ++rr) {
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        float t = a[rr][0].x * xr[m][0].x;
        t = fmaf(a[rr][0].y, xr[m][0].y, t); t = fmaf(a[rr][0].z, xr[m][0].z, t);
        t = fmaf(a[rr][0].w, xr[m][0].w, t); t = fmaf(a[rr][1].x, xr[m][1].x, t);
        t = fmaf(a[rr][1].y, xr[m][1].y, t); t = fmaf(a[rr][1].z, xr[m][1].z, t);
        t = fmaf(a[rr][1].w, xr[m][1].w, t);
        acc[rr * MB + m] = t;
      }
    }
    const float tot = warp_transpose_sum<float, NV>(acc);   // the warp's 256 columns, FP32
    if ((lane & ((1 << SH) - 1)) == 0) sred[warp][st][lane >> SH] = (double)tot;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < STEPS * NV; e += blockDim.x) {
    const int st = e / NV, v = e - st * NV;
    const int rr = v / MB, m = v - rr * MB;
    const int row = rbeg + st * kTileRpw + rr;
    if (row >= nb || m >= nm) continue;
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) s += sred[w][st][v];
    part[((size_t)blockIdx.x * nb + row) * MB + m] = s;
  }
}

// y[m * nb + r] = sum over slabs of member m's tile partials of row r.
__global__ void k_slab_sum_m(int nb, int nslab, int nm, int MB, const double *__restrict__ part,
                             double *__restrict__ y) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nb * nm) return;
  const int m = g / nb, r = g - m * nb;
  double s = 0.0;
  for (int sl = 0; sl < nslab; ++sl) s += part[((size_t)sl * nb + r) * MB + m];
  y[(size_t)m * nb + r] = s;
}

// ---- compensated ("double-float") BEM product: form 2 ----
// B = hi (FP32) + lo (BF16), x = xh + xl (FP32 pairs).  Per entry: the
// product hi * xh is split exactly with an FMA (p + e), the second-order
// terms hi * xl + lo * xh join e, p enters a TwoSum running sum S whose
// rounding errors are kept in C.  The result carries ~44 bits although
// every operation runs on the FP32 pipe (the film's potentials cancel
// ~50x in phi1 + phi2, so FP32 products alone lose 1e-5 there).
// __fmul_rn / __fadd_rn / __fsub_rn forbid contraction and reassociation.
// df_madd (the compensated multiply-add) is in nmg_internal.h: the adjoint's
// transpose product uses it too.

// (S, C) += (S2, C2) for FP32 pairs: TwoSum of the heads, the tails added.
__device__ __forceinline__ void df_add(float &S, float &C, float S2, float C2) {
  const float s2 = __fadd_rn(S, S2);
  const float bb = __fsub_rn(s2, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s2, bb)), __fsub_rn(S2, bb));
  S = s2;
  C = __fadd_rn(__fadd_rn(C, C2), err);
}

// warp_transpose_sum for NV (S, C) pairs, all in FP32 pair arithmetic: the
// FP64 pipe is used only for the one conversion per result afterwards.
template <int NV>
__device__ __forceinline__ void warp_transpose_sum_df(float (&S)[NV], float (&C)[NV]) {
  const int lane = threadIdx.x & 31;
  int n = NV;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (n > 1) {
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int i = 0; i < NV / 2; ++i) {
        if (i >= n / 2) break;
        const float sS = up ? S[i] : S[i + n / 2], sC = up ? C[i] : C[i + n / 2];
        const float kS = up ? S[i + n / 2] : S[i], kC = up ? C[i + n / 2] : C[i];
        const float rS = __shfl_xor_sync(0xffffffffu, sS, o), rC = __shfl_xor_sync(0xffffffffu, sC, o);
        S[i] = kS;
        C[i] = kC;
        df_add(S[i], C[i], rS, rC);
      }
      n >>= 1;
    } else {
      const float rS = __shfl_xor_sync(0xffffffffu, S[0], o), rC = __shfl_xor_sync(0xffffffffu, C[0], o);
      df_add(S[0], C[0], rS, rC);
    }
  }
}

__device__ __forceinline__ float bf16lo(unsigned w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16hi(unsigned w) { return __uint_as_float(w & 0xffff0000u); }

// x (nm members, member m at m * n) -> FP32 pairs xh + xl, zero-padded to ld.
__global__ void k_split_x(int n, int ld, int nm, const double *__restrict__ x, float *__restrict__ xh,
                          float *__restrict__ xl, const int *__restrict__ gate = nullptr) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ld * nm || (gate && !*gate)) return;
  const int m = g / ld, i = g - m * ld;
  const double v = i < n ? x[(size_t)m * n + i] : 0.0;
  const float h = (float)v;
  xh[g] = h;
  xl[g] = (float)(v - (double)h);
}

// One simulation: the warp-segment decomposition of k_gemv_f32 (8-column units).
__global__ void __launch_bounds__(kGemvThreads) k_gemv_df(int nb, int ld, long long seg, int maxr,
                                                           const float *__restrict__ Bh,
                                                           const uint16_t *__restrict__ Bl,
                                                           const float *__restrict__ xh,
                                                           const float *__restrict__ xl, double *__restrict__ part,
                                                           const int *__restrict__ gate = nullptr) {
  if (gate && !*gate) return;   // anchored product: the FP32 difference product runs instead
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long Q = ld / 8, total = (long long)nb * Q;
  const long long q0 = w * seg, q1 = min(total, q0 + seg);
  if (q0 >= q1) return;
  const long long rfirst = q0 / Q;
  for (long long r = rfirst; r * Q < q1; ++r) {
    const long long a = max(q0, r * Q), e = min(q1, (r + 1) * Q);
    const float *rh = Bh + r * (long long)ld;
    const uint16_t *rl = Bl + r * (long long)ld;
    float S = 0.f, C = 0.f;
    for (long long q = a + lane; q < e; q += 32) {
      const long long c = 8 * (q - r * Q);
      const float4 h0 = __ldcs(reinterpret_cast<const float4 *>(rh + c));
      const float4 h1 = __ldcs(reinterpret_cast<const float4 *>(rh + c) + 1);
      const uint4 lq = __ldcs(reinterpret_cast<const uint4 *>(rl + c));
      const float4 a0 = __ldg(reinterpret_cast<const float4 *>(xh + c));
      const float4 a1 = __ldg(reinterpret_cast<const float4 *>(xh + c) + 1);
      const float4 b0 = __ldg(reinterpret_cast<const float4 *>(xl + c));
      const float4 b1 = __ldg(reinterpret_cast<const float4 *>(xl + c) + 1);
      df_madd(h0.x, bf16lo(lq.x), a0.x, b0.x, S, C);
      df_madd(h0.y, bf16hi(lq.x), a0.y, b0.y, S, C);
      df_madd(h0.z, bf16lo(lq.y), a0.z, b0.z, S, C);
      df_madd(h0.w, bf16hi(lq.y), a0.w, b0.w, S, C);
      df_madd(h1.x, bf16lo(lq.z), a1.x, b1.x, S, C);
      df_madd(h1.y, bf16hi(lq.z), a1.y, b1.y, S, C);
      df_madd(h1.z, bf16lo(lq.w), a1.z, b1.z, S, C);
      df_madd(h1.w, bf16hi(lq.w), a1.w, b1.w, S, C);
    }
    const double sum = warp_sum((double)S + (double)C);
    if (lane == 0) part[w * maxr + (r - rfirst)] = sum;
  }
}

// Ensemble: tiles of kDfCols columns x kDfRows rows; the slab's xh / xl of
// every member in shared memory, each warp kDfRpw rows at a time.
constexpr int kDfCols = 512, kDfRows = 64, kDfRpw = 2;

template <int MB>
__global__ void __launch_bounds__(256) k_gemm_df(int nb, int ld, int nm, const float *__restrict__ Bh,
                                                 const uint16_t *__restrict__ Bl, const float *__restrict__ xh,
                                                 const float *__restrict__ xl, double *__restrict__ part,
                                                 const int *__restrict__ gate = nullptr) {
  if (gate && !*gate) return;   // anchored product: the FP32 difference product runs instead
  __shared__ float4 sh[MB][kDfCols / 4], sl[MB][kDfCols / 4];
  const int slab = blockIdx.x, c0 = slab * kDfCols;
  const int ncol = min(kDfCols, ld - c0);   // a multiple of 8
  for (int i = threadIdx.x; i < MB * (kDfCols / 4); i += blockDim.x) {
    const int m = i / (kDfCols / 4), q = i - m * (kDfCols / 4);
    const bool ok = m < nm && 4 * q < ncol;
    sh[m][q] = ok ? __ldg(reinterpret_cast<const float4 *>(xh + (size_t)m * ld + c0) + q) : make_float4(0.f, 0.f, 0.f, 0.f);
    sl[m][q] = ok ? __ldg(reinterpret_cast<const float4 *>(xl + (size_t)m * ld + c0) + q) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int units = ncol / 8;
  const int rend = min(nb, (int)(blockIdx.y + 1) * kDfRows);
  for (int r0 = blockIdx.y * kDfRows + warp * kDfRpw; r0 < rend; r0 += 8 * kDfRpw) {
    float S[kDfRpw * MB], C[kDfRpw * MB];
#pragma unroll
    for (int q = 0; q < kDfRpw * MB; ++q) S[q] = C[q] = 0.f;
    for (int u = lane; u < units; u += 32) {
      float hv[kDfRpw][8], lv[kDfRpw][8];
#pragma unroll
      for (int rr = 0; rr < kDfRpw; ++rr) {
        const size_t off = (size_t)min(r0 + rr, nb - 1) * ld + c0 + 8 * u;
        const float4 h0 = __ldcs(reinterpret_cast<const float4 *>(Bh + off));
        const float4 h1 = __ldcs(reinterpret_cast<const float4 *>(Bh + off) + 1);
        const uint4 lq = __ldcs(reinterpret_cast<const uint4 *>(Bl + off));
        hv[rr][0] = h0.x; hv[rr][1] = h0.y; hv[rr][2] = h0.z; hv[rr][3] = h0.w;
        hv[rr][4] = h1.x; hv[rr][5] = h1.y; hv[rr][6] = h1.z; hv[rr][7] = h1.w;
        lv[rr][0] = bf16lo(lq.x); lv[rr][1] = bf16hi(lq.x); lv[rr][2] = bf16lo(lq.y); lv[rr][3] = bf16hi(lq.y);
        lv[rr][4] = bf16lo(lq.z); lv[rr][5] = bf16hi(lq.z); lv[rr][6] = bf16lo(lq.w); lv[rr][7] = bf16hi(lq.w);
      }
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const float4 a0 = sh[m][2 * u], a1 = sh[m][2 * u + 1], b0 = sl[m][2 * u], b1 = sl[m][2 * u + 1];
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int rr = 0; rr < kDfRpw; ++rr)
#pragma unroll
          for (int j = 0; j < 8; ++j) df_madd(hv[rr][j], lv[rr][j], av[j], bv[j], S[rr * MB + m], C[rr * MB + m]);
      }
    }
    constexpr int NV = kDfRpw * MB;
    constexpr int SH = NV >= 32 ? 0 : (NV >= 16 ? 1 : (NV >= 8 ? 2 : 3));
    warp_transpose_sum_df<NV>(S, C);
    const int v = lane >> SH;
    const int rr = v / MB, m = v - rr * MB;
    if ((lane & ((1 << SH) - 1)) == 0 && m < nm && r0 + rr < nb)
      part[((size_t)slab * nb + r0 + rr) * MB + m] = (double)S[0] + (double)C[0];
  }
}

// y[m * nb + r] = ordered sum of member m's partials of row r.
__global__ void k_row_sum_m(int nb, long long Q, long long seg, int maxr, long long nwarps, int nm, int MB,
                            const double *__restrict__ part, double *__restrict__ y) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nb * nm) return;
  const int m = g / nb, r = g - m * nb;
  const long long w0 = ((long long)r * Q) / seg, w1 = min(nwarps - 1, ((long long)(r + 1) * Q - 1) / seg);
  double s = 0.0;
  for (long long w = w0; w <= w1; ++w) s += part[(w * maxr + (r - (w * seg) / Q)) * MB + m];
  y[(size_t)m * nb + r] = s;
}

// ---- anchored BEM product (compensated form) ----
// y = B x is formed as y0 + B32 (x - x0), where (x0, y0 = B x0) is the chunk's
// last compensated product (the anchor) and B32 the FP32 part of the matrix.
// The FP32 product's rounding error is ~2^-24 |B| |x - x0| instead of
// 2^-24 |B| |x|, so while x stays within tol of x0 (max norm, per member) the
// result keeps (tol x the FP32 error), and the matrix is read at 4 B per entry
// on an HBM-bound kernel instead of 6 B on an FP32-pipe-bound one.  Every
// product is computed from its own x; the anchor is a second solution of the
// same linear map that the difference is added to.
//
// k_anchor_drift: d = FP32(x - x0) zero-padded to ld (the FP32 kernels' x
// layout) and per-member maxima of |x - x0| and |x| (bit patterns of
// non-negative doubles order like the values; NaN orders above +inf).
__global__ void k_anchor_drift(int n, int ld, int nm, const double *__restrict__ x, const double *__restrict__ x0,
                               float *__restrict__ d, unsigned long long *__restrict__ mx) {
  __shared__ unsigned long long smx[2 * kChunk];
  if (threadIdx.x < 2 * kChunk) smx[threadIdx.x] = 0ull;
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < ld * nm) {
    const int m = g / ld, i = g - m * ld;
    float dv = 0.f;
    if (i < n) {
      const double v = x[(size_t)m * n + i], e = v - x0[(size_t)m * n + i];
      dv = (float)e;
      atomicMax(&smx[m], (unsigned long long)__double_as_longlong(fabs(e)));
      atomicMax(&smx[kChunk + m], (unsigned long long)__double_as_longlong(fabs(v)));
    }
    d[g] = dv;
  }
  __syncthreads();
  if (threadIdx.x < 2 * kChunk && smx[threadIdx.x]) atomicMax(&mx[threadIdx.x], smx[threadIdx.x]);
}

// One thread: refresh (flag = 1) when the chunk has no anchor yet or a
// member drifted past tol; clears the maxima for the next chunk and counts
// products / refreshes.
__global__ void k_anchor_decide(int nm, double tol, unsigned long long *__restrict__ mx, const int *__restrict__ valid,
                                int *__restrict__ flag, long long *__restrict__ count, float *__restrict__ scale = nullptr) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int refresh = *valid ? 0 : 1;
  for (int m = 0; m < nm; ++m) {
    const double dm = __longlong_as_double((long long)mx[m]), xm = __longlong_as_double((long long)mx[kChunk + m]);
    if (!(dm <= tol * xm)) refresh = 1;
    if (scale) {   // FP16 fragment product: 2^k with max|x - x0| 2^k in [2^13, 2^14)
      int e = 0;
      if (dm > 0.0 && dm <= 1e300) frexp(dm, &e);
      e = max(-100, min(100, e));
      scale[m] = (float)ldexp(1.0, 14 - e);
    }
  }
  for (int k = 0; k < 2 * kChunk; ++k) mx[k] = 0ull;
  *flag = refresh;
  count[0] += 1;
  count[1] += refresh;
}

// Ensemble epilogue: sum the slab partials of whichever product ran (the
// compensated one has nslab_df slabs, the FP32 one nslab_32), then either
// store the new anchor or add the difference product to the old one.
__global__ void k_anchor_slab_sum(int nb, int nslab_df, int nslab_32, int nm, int MB, const double *__restrict__ part,
                                  const int *__restrict__ flag, int *__restrict__ valid, const double *__restrict__ x,
                                  double *__restrict__ x0, double *__restrict__ y0, double *__restrict__ y) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int refresh = *flag;
  if (g == 0 && refresh) *valid = 1;
  if (g >= nb * nm) return;
  const int m = g / nb, r = g - m * nb;
  const int nslab = refresh ? nslab_df : nslab_32;
  double s = 0.0;
  for (int sl = 0; sl < nslab; ++sl) s += part[((size_t)sl * nb + r) * MB + m];
  const size_t o = (size_t)m * nb + r;
  if (refresh) {
    y0[o] = s;
    x0[o] = x[o];
    y[o] = s;
  } else {
    y[o] = y0[o] + s;
  }
}

// ---- anchored ensemble product, FP16 fragment form ----
// The difference product B (x - x0) of 8 members on the tensor cores:
// mma.m16n8k16 with B's 16 x 16 tiles as the A operand (FP16, stored in
// fragment order by k_pack_bem16f, scaled by 2^sB), the members' x - x0 as
// the 16 x 8 B operand (FP16, scaled per member by 2^sX), FP32 accumulation.
// One 16-byte load per lane and tile and one mma per tile replace 128 FP32
// FMAs per lane, so the 2-byte matrix streams at the memory rate.
//
// k_pack_x16f: x - x0 (FP32, [member][ld]) times the member scales in the
// B-operand fragment order: k-tile kb, lane 4 n + t holds rows 2t, 2t+1,
// 2t+8, 2t+9 of column n (member n; 0 beyond nm or nb).
__global__ void k_pack_x16f(int nb, int ld, int nm, int KT, const float *__restrict__ xh,
                            const float *__restrict__ scale, uint2 *__restrict__ out, const int *__restrict__ gate) {
  if (gate && *gate) return;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= KT * 32) return;
  const int kb = g >> 5, lane = g & 31, n = lane >> 2, t = lane & 3;
  const float sc = n < nm ? scale[n] : 0.f;
  unsigned w[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    float v[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = 16 * kb + 2 * t + h + 8 * j;
      v[h] = (n < nm && k < nb) ? xh[(size_t)n * ld + k] * sc : 0.f;
    }
    const __half2 p = __floats2half2_rn(v[0], v[1]);
    memcpy(&w[j], &p, sizeof(unsigned));
  }
  out[g] = make_uint2(w[0], w[1]);
}

// k_gemm_h16mma: warp w streams tiles [w seg, (w+1) seg) of the row-block-
// major tile sequence (KT tiles per row block), kH16Unroll tiles of loads in
// flight, and stores its 16 x 8 accumulator (C-fragment order, a float4 per
// lane) whenever the row block changes: part[(w maxr + local block) 32 + lane].
constexpr int kH16Unroll = 8;
__global__ void __launch_bounds__(256) k_gemm_h16mma(long long TT, int KT, long long seg, int maxr,
                                                     const uint4 *__restrict__ A, const uint2 *__restrict__ X,
                                                     float4 *__restrict__ part, const int *__restrict__ gate) {
  if (gate && *gate) return;
  const int lane = threadIdx.x & 31;
  const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long t0 = w * seg, t1 = min(t0 + seg, TT);
  if (t0 >= t1) return;   // warp-uniform
  const int rfirst = (int)(t0 / KT);
  int cur = rfirst, lrb = rfirst, lkb = (int)(t0 - (long long)rfirst * KT);
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
  for (long long tb = t0; tb < t1; tb += kH16Unroll) {
    uint4 a[kH16Unroll];
    uint2 b[kH16Unroll];
    int rbu[kH16Unroll];
#pragma unroll
    for (int u = 0; u < kH16Unroll; ++u) {
      const bool in = tb + u < t1;
      rbu[u] = lrb;
      a[u] = in ? __ldcs(A + (tb + u) * 32 + lane) : make_uint4(0u, 0u, 0u, 0u);
      b[u] = in ? __ldg(X + (size_t)lkb * 32 + lane) : make_uint2(0u, 0u);
      if (++lkb == KT) { lkb = 0; ++lrb; }
    }
#pragma unroll
    for (int u = 0; u < kH16Unroll; ++u) {
      if (tb + u < t1) {   // warp-uniform
        if (rbu[u] != cur) {
          part[((size_t)w * maxr + (cur - rfirst)) * 32 + lane] = make_float4(c0, c1, c2, c3);
          c0 = c1 = c2 = c3 = 0.f;
          cur = rbu[u];
        }
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(c0), "+f"(c1), "+f"(c2), "+f"(c3)
            : "r"(a[u].x), "r"(a[u].y), "r"(a[u].z), "r"(a[u].w), "r"(b[u].x), "r"(b[u].y));
      }
    }
  }
  part[((size_t)w * maxr + (cur - rfirst)) * 32 + lane] = make_float4(c0, c1, c2, c3);
}

// Ensemble epilogue of the FP16 fragment form: on a refresh, the compensated
// product's slab partials (as k_anchor_slab_sum); otherwise row r of member m
// sums its row block's partials over the warps that streamed it, in warp
// order (element (r mod 16, m) of the C fragment: lane 4 (r mod 8) + m/2,
// component 2 [r mod 16 >= 8] + m mod 2), undoes the two scales and adds y0.
__global__ void k_anchor_h16_sum(int nb, int nslab_df, int nm, int MB, const double *__restrict__ part_df,
                                 const float *__restrict__ part16, int KT, long long seg, int maxr, long long nwarps,
                                 double inv_scale_b, const float *__restrict__ scale_x, const int *__restrict__ flag,
                                 int *__restrict__ valid, const double *__restrict__ x, double *__restrict__ x0,
                                 double *__restrict__ y0, double *__restrict__ y) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int refresh = *flag;
  if (g == 0 && refresh) *valid = 1;
  if (g >= nb * nm) return;
  const int m = g / nb, r = g - m * nb;
  const size_t o = (size_t)m * nb + r;
  if (refresh) {
    double s = 0.0;
    for (int sl = 0; sl < nslab_df; ++sl) s += part_df[((size_t)sl * nb + r) * MB + m];
    y0[o] = s;
    x0[o] = x[o];
    y[o] = s;
    return;
  }
  const int rb = r >> 4, rr = r & 15;
  const int lane = (rr & 7) * 4 + (m >> 1), comp = (rr >= 8 ? 2 : 0) + (m & 1);
  const long long w0 = ((long long)rb * KT) / seg, w1 = min(nwarps - 1, ((long long)(rb + 1) * KT - 1) / seg);
  double s = 0.0;
  for (long long w = w0; w <= w1; ++w) {
    const long long loc = rb - (w * seg) / KT;
    s += (double)part16[(((size_t)w * maxr + loc) * 32 + lane) * 4 + comp];
  }
  y[o] = y0[o] + s * (inv_scale_b / (double)scale_x[m]);
}

// One simulation: k_row_sum over the shared segment partials (the compensated
// and FP32 single products use the same decomposition), then the anchor step.
__global__ void k_anchor_row_sum(int nb, long long Q, long long seg, int maxr, long long nwarps,
                                 const double *__restrict__ part, const int *__restrict__ flag,
                                 int *__restrict__ valid, const double *__restrict__ x, double *__restrict__ x0,
                                 double *__restrict__ y0, double *__restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int refresh = *flag;
  if (r == 0 && refresh) *valid = 1;
  if (r >= nb) return;
  const long long w0 = (r * Q) / seg, w1 = min(nwarps - 1, ((r + 1) * Q - 1) / seg);
  double s = 0.0;
  for (long long w = w0; w <= w1; ++w) s += part[w * maxr + (r - (w * seg) / Q)];
  if (refresh) {
    y0[r] = s;
    x0[r] = x[r];
    y[r] = s;
  } else {
    y[r] = y0[r] + s;
  }
}

// Dirichlet right-hand side (op_load_DBC, sign folded): interior rows
// -sum_{j boundary} K_ij phi2b_j, boundary rows phi2b; boundary values of the
// warm start are set to phi2b.
__global__ void k_dbc_rhs(int N, const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                          const double *__restrict__ K, const int32_t *__restrict__ b_of_node,
                          const double *__restrict__ phi2b_all, double *__restrict__ rhs, double *__restrict__ phi2,
                          int nb = 0, int nrep = 1) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)N * nrep) return;
  const int mbr = (int)(g / N), i = (int)(g - (long long)mbr * N);
  const double *phi2b = phi2b_all + (size_t)mbr * nb;
  int bi = b_of_node[i];
  if (bi >= 0) { rhs[g] = phi2b[bi]; phi2[g] = phi2b[bi]; return; }
  double s = 0.0;
  for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
    int b = b_of_node[col_idx[k]];
    if (b >= 0) s += K[k] * phi2b[b];
  }
  rhs[g] = -s;
}

__global__ void k_add(int n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ c) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] + b[i];
}

// Anisotropy field from its polynomial form (nsim_anisotropy.ml:143-206: the
// tangential gradient -(1/mu0 Ms)(grad E - (m.grad E) m) expanded into
// monomials by the host): H_d = sum_t c_{t,d} m^{p_t}, written to h (3 per
// node, all members).  The term table is read uniformly by every thread.
__global__ void k_anis_poly(long long n, const double *__restrict__ m, int nt, const int32_t *__restrict__ pw,
                            const double *__restrict__ c, double *__restrict__ h) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double px[kAnisMaxPow + 1], py[kAnisMaxPow + 1], pz[kAnisMaxPow + 1];
  anis_powers(m[3 * i], m[3 * i + 1], m[3 * i + 2], px, py, pz);
  double h0 = 0.0, h1 = 0.0, h2 = 0.0;
  for (int t = 0; t < nt; ++t) {
    const double mono = anis_monomial(__ldg(pw + t), px, py, pz);
    h0 = fma(__ldg(c + 3 * t), mono, h0);
    h1 = fma(__ldg(c + 3 * t + 1), mono, h1);
    h2 = fma(__ldg(c + 3 * t + 2), mono, h2);
  }
  h[3 * i] = h0; h[3 * i + 1] = h1; h[3 * i + 2] = h2;
}

// dm_dcurrent = (J . grad) m (program set_dm_dcurrent, nmag_lam.py:872-903):
// op_grad_m = <grad_m(i,j)||d/dxj m(i)> is G_j applied to m_i (the pattern
// and values of op_grad_phi without its sign), then site-wise
// grad_m(i,j) current_density(j) summed over j in order, then CFBOX.
__global__ void k_stt_dmdc(int N, int nrep, int nnz, const int32_t *__restrict__ row_ptr,
                           const int32_t *__restrict__ col_idx, const double *__restrict__ G,
                           const double *__restrict__ ivol, const double *__restrict__ m,
                           const double *__restrict__ J, double *__restrict__ out) {
  const long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gi >= (long long)N * nrep) return;
  const int mbr = (int)(gi / N), i = (int)(gi - (long long)mbr * N);
  const double *mm = m + (size_t)mbr * 3 * N;
  double g[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};   // g[comp][direction]
  for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
    const double gx = G[k], gy = G[(size_t)nnz + k], gz = G[2 * (size_t)nnz + k];
    const double *mj = mm + 3 * (size_t)col_idx[k];
    for (int c = 0; c < 3; ++c) {
      g[c][0] += gx * mj[c]; g[c][1] += gy * mj[c]; g[c][2] += gz * mj[c];
    }
  }
  const double *jp = J + 3 * (size_t)gi;
  const double iv = ivol[i];
  for (int c = 0; c < 3; ++c) out[3 * (size_t)gi + c] = ((g[c][0] * jp[0] + g[c][1] * jp[1]) + g[c][2] * jp[2]) * iv;
}

struct NodeArgs {
  int N, nnz, do_demag, nrep;   // nrep members: m, h_ext and outputs member-major (3N each), phi N each
  const int32_t *row_ptr, *col_idx;
  const double *K, *G, *ivol, *m, *phi, *h_ext;   // ivol: 1 / box volume
  const double *anis_node;   // per-node anisotropy coefficient (element parameters) or null
  const double *anis_in;     // polynomial anisotropy field (3 per node, all members) or null
  const double *dmdc;        // spin-transfer dm_dcurrent (3 per node, all members) or null
  const double *pin;         // per-node factor of dm/dt (one per node, shared by members) or null
  double C4, C5;             // its LLG coefficients
  double c_exch, C1, C2, C3, K1, anis, ax, ay, az;
  double *h_exch, *h_demag, *h_anis, *h_total, *dmdt;
};

// Fused node kernel: the two SpMV epilogues and every site-wise equation.
__global__ void k_heff_llg(NodeArgs a) {
  const long long gi = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (gi >= (long long)a.N * a.nrep) return;
  const int mbr = (int)(gi / a.N), i = (int)(gi - (long long)mbr * a.N);
  const double *mm = a.m + (size_t)mbr * 3 * a.N;
  const double *ph = a.do_demag ? a.phi + (size_t)mbr * a.N : a.phi;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
  const int lo = a.row_ptr[i], hi = a.row_ptr[i + 1];
  for (int k = lo; k < hi; ++k) {
    const int j = a.col_idx[k];
    const double kv = a.K[k];
    const double *mj = mm + 3 * (size_t)j;
    s0 += kv * mj[0]; s1 += kv * mj[1]; s2 += kv * mj[2];
    if (a.do_demag) {
      const double pj = ph[j];
      g0 += a.G[k] * pj; g1 += a.G[(size_t)a.nnz + k] * pj; g2 += a.G[2 * (size_t)a.nnz + k] * pj;
    }
  }
  const double iv = a.ivol[i];
  const double ce = -a.c_exch * iv;
  const double hx[3] = {ce * s0, ce * s1, ce * s2};
  const double hd[3] = {-g0 * iv, -g1 * iv, -g2 * iv};
  const double *m = mm + 3 * (size_t)i;
  double ha[3] = {0.0, 0.0, 0.0};
  if (a.anis_in) {
    const double *p = a.anis_in + 3 * (size_t)gi;
    ha[0] = p[0]; ha[1] = p[1]; ha[2] = p[2];
  }
  if (a.K1 != 0.0 || a.anis_node) {
    const double c = a.anis_node ? a.anis_node[i] : a.anis;
    double am = (a.ax * m[0] + a.ay * m[1]) + a.az * m[2];
    ha[0] += c * am * (a.ax - am * m[0]);
    ha[1] += c * am * (a.ay - am * m[1]);
    ha[2] += c * am * (a.az - am * m[2]);
  }
  const double *he = a.h_ext + 3 * (size_t)gi;
  double H[3];
  for (int d = 0; d < 3; ++d) H[d] = ((he[d] + hx[d]) + ha[d]) + hd[d];
  const double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
  const double mxmxH[3] = {m[1] * mxH[2] - m[2] * mxH[1], m[2] * mxH[0] - m[0] * mxH[2],
                           m[0] * mxH[1] - m[1] * mxH[0]};
  const double c3 = a.C3 * (1.0 - ((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]));
  double f[3];
  for (int d = 0; d < 3; ++d) f[d] = (a.C1 * mxH[d] + a.C2 * mxmxH[d]) + c3 * m[d];
  if (a.dmdc) {   // + C4 m x (m x dm_dcurrent) + C5 m x dm_dcurrent (nmag_lam.py:417-424)
    const double *u = a.dmdc + 3 * (size_t)gi;
    const double mxu[3] = {m[1] * u[2] - m[2] * u[1], m[2] * u[0] - m[0] * u[2], m[0] * u[1] - m[1] * u[0]};
    const double mxmxu[3] = {m[1] * mxu[2] - m[2] * mxu[1], m[2] * mxu[0] - m[0] * mxu[2],
                             m[0] * mxu[1] - m[1] * mxu[0]};
    for (int d = 0; d < 3; ++d) f[d] = (f[d] + a.C4 * mxmxu[d]) + a.C5 * mxu[d];
  }
  if (a.pin) {   // every LLG term carries the factor pin (nmag_lam.py:417-424)
    const double p = a.pin[i];
    for (int d = 0; d < 3; ++d) f[d] *= p;
  }
  for (int d = 0; d < 3; ++d) {
    const size_t o = 3 * (size_t)gi + d;
    a.h_exch[o] = hx[d]; a.h_demag[o] = hd[d]; a.h_anis[o] = ha[d]; a.h_total[o] = H[d];
    a.dmdt[o] = f[d];
  }
}

// Energy densities (nmag_lam.py:454-460): E_exch, E_demag, E_ext, E_anis, E_total.
__global__ void k_energy(int N, const double *__restrict__ m, const double *__restrict__ hx,
                         const double *__restrict__ hd, const double *__restrict__ he, double ch, double ce,
                         double K1, double ax, double ay, double az, int ne, const int32_t *__restrict__ epow,
                         const double *__restrict__ ecoef, double *__restrict__ E) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double *mi = m + 3 * (size_t)i, *x = hx + 3 * (size_t)i, *d = hd + 3 * (size_t)i, *e = he + 3 * (size_t)i;
  double ex = ch * ((mi[0] * x[0] + mi[1] * x[1]) + mi[2] * x[2]);
  double dm = ch * ((mi[0] * d[0] + mi[1] * d[1]) + mi[2] * d[2]);
  double ez = ce * ((mi[0] * e[0] + mi[1] * e[1]) + mi[2] * e[2]);
  double an = 0.0;
  if (K1 != 0.0) { double am = (ax * mi[0] + ay * mi[1]) + az * mi[2]; an = -K1 * am * am; }
  if (ne > 0) {   // polynomial energy density E_anis = sum_t e_t m^{p_t}
    double px[kAnisMaxPow + 1], py[kAnisMaxPow + 1], pz[kAnisMaxPow + 1];
    anis_powers(mi[0], mi[1], mi[2], px, py, pz);
    for (int t = 0; t < ne; ++t) an = fma(__ldg(ecoef + t), anis_monomial(__ldg(epow + t), px, py, pz), an);
  }
  E[i] = ex; E[N + i] = dm; E[2 * (size_t)N + i] = ez; E[3 * (size_t)N + i] = an;
  E[4 * (size_t)N + i] = ((dm + ex) + ez) + an;
}

// Block partial sums of V_i, V_i m_i (3) and V_i E_k,i (5): 9 columns.
__global__ void k_avg_partials(int N, const double *__restrict__ m, const double *__restrict__ vol,
                               const double *__restrict__ E, double *__restrict__ part, size_t estride) {
  __shared__ double smem[32 * 9];
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double V = vol[i];
    v[0] += V;
    for (int d = 0; d < 3; ++d) v[1 + d] += V * m[3 * (size_t)i + d];
    if (E) for (int k = 0; k < 5; ++k) v[4 + k] += V * E[(size_t)k * estride + i];
  }
  block_sum<9>(v, smem);
  if (threadIdx.x == 0) for (int j = 0; j < 9; ++j) part[9 * blockIdx.x + j] = v[j];
}

__global__ void k_maxdm_partials(int N, const double *__restrict__ a, const double *__restrict__ b,
                                 double *__restrict__ part) {
  __shared__ double smem[32];
  double mx = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double d0 = a[3 * (size_t)i] - b[3 * (size_t)i], d1 = a[3 * (size_t)i + 1] - b[3 * (size_t)i + 1],
           d2 = a[3 * (size_t)i + 2] - b[3 * (size_t)i + 2];
    mx = fmax(mx, sqrt(d0 * d0 + d1 * d1 + d2 * d2));
  }
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, smem[w]);
    part[blockIdx.x] = r;
  }
}

// Solver ordering and two-level data, built once on the host:
//  * nodes sorted by spatial bin (Morton order of bins sized for ~kAgg nodes),
//    so that kAgg consecutive solver rows form a compact aggregate and each
//    256-row CG block holds 4 whole aggregates;
//  * the CSR of K in that order (columns sorted);
//  * the aggregated operator A_c = P^T K P (P: piecewise-constant
//    prolongation), regularised by (mean diagonal / nc) 1 1^T for the
//    constant null space, inverted densely (Cholesky).  Skipped for more
//    than kMaxCoarse aggregates or when the options disable it.
constexpr int kMaxCoarse = 2048;

uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  auto spread = [](uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
  };
  return spread(x) | spread(y) << 1 | spread(z) << 2;
}

int build_cg_ordering(nmg_handle *h, std::string &err) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const int N = M.N, nnz = M.nnz;
  std::vector<int32_t> rp(N + 1), ci(nnz), bon(N);
  std::vector<double> K(nnz), X(3 * (size_t)N);
  NMG_CUDA_TRY(cudaMemcpy(rp.data(), M.row_ptr.p, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost), "d2h");
  NMG_CUDA_TRY(cudaMemcpy(ci.data(), M.col_idx.p, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost), "d2h");
  NMG_CUDA_TRY(cudaMemcpy(K.data(), M.K.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost), "d2h");
  NMG_CUDA_TRY(cudaMemcpy(X.data(), M.coords.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost), "d2h");
  NMG_CUDA_TRY(cudaMemcpy(bon.data(), M.b_of_node.p, sizeof(int32_t) * N, cudaMemcpyDeviceToHost), "d2h");
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) { lo[d] = X[d]; hi[d] = X[d]; }
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], X[3 * i + d]); hi[d] = std::max(hi[d], X[3 * i + d]); }
  double vol = 1.0;
  for (int d = 0; d < 3; ++d) vol *= std::max(hi[d] - lo[d], 1e-30);
  const double H = std::cbrt(vol * kAgg / N);
  std::vector<std::pair<uint64_t, int>> key(N);
  for (int i = 0; i < N; ++i) {
    uint32_t b[3];
    for (int d = 0; d < 3; ++d) b[d] = (uint32_t)std::min(2097151.0, std::floor((X[3 * i + d] - lo[d]) / H));
    key[i] = {morton3(b[0], b[1], b[2]), i};
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> perm(N), inv(N), prow(N + 1), pcol(nnz), pbnd(N);
  std::vector<double> pK(nnz);
  for (int r = 0; r < N; ++r) { perm[r] = key[r].second; inv[key[r].second] = r; }
  prow[0] = 0;
  std::vector<std::pair<int32_t, double>> row;
  for (int r = 0; r < N; ++r) {
    const int node = perm[r];
    row.clear();
    for (int k = rp[node]; k < rp[node + 1]; ++k) row.push_back({inv[ci[k]], K[k]});
    std::sort(row.begin(), row.end(), [](const std::pair<int32_t, double> &x, const std::pair<int32_t, double> &y) {
      return x.first < y.first;
    });
    int o = prow[r];
    for (auto &e : row) { pcol[o] = e.first; pK[o] = e.second; ++o; }
    prow[r + 1] = o;
    pbnd[r] = bon[node] >= 0 ? 1 : 0;
  }
  NMG_CUDA_TRY(W.perm.alloc(N), "alloc");
  NMG_CUDA_TRY(W.prow.alloc(N + 1), "alloc");
  NMG_CUDA_TRY(W.pcol.alloc(nnz), "alloc");
  NMG_CUDA_TRY(W.pbnd.alloc(N), "alloc");
  NMG_CUDA_TRY(W.pK.alloc(nnz), "alloc");
  NMG_CUDA_TRY(W.xperm.alloc((size_t)N * ((h->nrep > 1 || h->mixed_cg()) ? kChunk : 1)), "alloc");
  NMG_CUDA_TRY(W.z32.alloc((size_t)N * kChunk), "alloc");
  NMG_CUDA_TRY(cudaMemcpy(W.perm.p, perm.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "h2d");
  NMG_CUDA_TRY(cudaMemcpy(W.prow.p, prow.data(), sizeof(int32_t) * (N + 1), cudaMemcpyHostToDevice), "h2d");
  NMG_CUDA_TRY(cudaMemcpy(W.pcol.p, pcol.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice), "h2d");
  NMG_CUDA_TRY(cudaMemcpy(W.pbnd.p, pbnd.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "h2d");
  NMG_CUDA_TRY(cudaMemcpy(W.pK.p, pK.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice), "h2d");
  if (h->mixed_cg()) {
    // the mixed-precision CG's shared-memory row order, made once here: in each
    // row the columns inside the block's row range (kCGThreads rows) first, by
    // the same swaps the kernel would make; mode 1 zeroes boundary columns
    std::vector<int32_t> mcol(pcol), mmid(N, 0);
    std::vector<double> mK0(pK), mK1(nnz);
    for (int k = 0; k < nnz; ++k) mK1[k] = 0.0;
    for (int r = 0; r < N; ++r) {
      const int row0 = (r / kCGThreads) * kCGThreads;
      for (int k = prow[r]; k < prow[r + 1]; ++k) mK1[k] = pbnd[pcol[k]] ? 0.0 : pK[k];
      int mid = prow[r];
      for (int k = prow[r]; k < prow[r + 1]; ++k) {
        const int j = mcol[k];
        if (j >= row0 && j < row0 + kCGThreads) {
          if (k != mid) {
            std::swap(mcol[mid], mcol[k]);
            std::swap(mK0[mid], mK0[k]);
            std::swap(mK1[mid], mK1[k]);
          }
          ++mid;
        }
      }
      mmid[r] = mid - prow[r];
    }
    std::vector<float> m32(2 * (size_t)nnz);
    for (int k = 0; k < nnz; ++k) { m32[k] = (float)mK0[k]; m32[nnz + (size_t)k] = (float)mK1[k]; }
    NMG_CUDA_TRY(W.mcol.alloc(nnz), "alloc");
    NMG_CUDA_TRY(W.mmid.alloc(N), "alloc");
    NMG_CUDA_TRY(W.mK.alloc(2 * (size_t)nnz), "alloc");
    NMG_CUDA_TRY(W.mK32.alloc(2 * (size_t)nnz), "alloc");
    NMG_CUDA_TRY(cudaMemcpy(W.mcol.p, mcol.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice), "h2d");
    NMG_CUDA_TRY(cudaMemcpy(W.mmid.p, mmid.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "h2d");
    NMG_CUDA_TRY(cudaMemcpy(W.mK.p, mK0.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice), "h2d");
    NMG_CUDA_TRY(cudaMemcpy(W.mK.p + nnz, mK1.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice), "h2d");
    NMG_CUDA_TRY(cudaMemcpy(W.mK32.p, m32.data(), sizeof(float) * 2 * nnz, cudaMemcpyHostToDevice), "h2d");
  }
  W.nc = 0;
  const int nc = (N + kAgg - 1) / kAgg;
  if (h->opt.cg_no_coarse || nc > kMaxCoarse || nc < 2) return 0;
  std::vector<double> A((size_t)nc * nc, 0.0);
  for (int r = 0; r < N; ++r)
    for (int k = prow[r]; k < prow[r + 1]; ++k) A[(size_t)(r / kAgg) * nc + pcol[k] / kAgg] += pK[k];
  double md = 0.0;
  for (int I = 0; I < nc; ++I) md += A[(size_t)I * nc + I];
  md /= nc;
  for (auto &v : A) v += md / nc;
  // Cholesky A = L L^T (lower, in place), then A^-1 = L^-T L^-1
  for (int j = 0; j < nc; ++j) {
    double d = A[(size_t)j * nc + j];
    for (int k = 0; k < j; ++k) d -= A[(size_t)j * nc + k] * A[(size_t)j * nc + k];
    if (!(d > 0.0)) return 0;   // not positive definite: run without the coarse level
    d = std::sqrt(d);
    A[(size_t)j * nc + j] = d;
    for (int i = j + 1; i < nc; ++i) {
      double s = A[(size_t)i * nc + j];
      for (int k = 0; k < j; ++k) s -= A[(size_t)i * nc + k] * A[(size_t)j * nc + k];
      A[(size_t)i * nc + j] = s / d;
    }
  }
  std::vector<double> Linv((size_t)nc * nc, 0.0), Ainv((size_t)nc * nc, 0.0);
  for (int j = 0; j < nc; ++j) {   // column j of L^-1 by forward substitution
    for (int i = j; i < nc; ++i) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int k = j; k < i; ++k) s -= A[(size_t)i * nc + k] * Linv[(size_t)k * nc + j];
      Linv[(size_t)i * nc + j] = s / A[(size_t)i * nc + i];
    }
  }
  for (int i = 0; i < nc; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int k = i; k < nc; ++k) s += Linv[(size_t)k * nc + i] * Linv[(size_t)k * nc + j];
      Ainv[(size_t)i * nc + j] = s;
      Ainv[(size_t)j * nc + i] = s;
    }
  NMG_CUDA_TRY(W.ainv.alloc((size_t)nc * nc), "alloc coarse inverse");
  NMG_CUDA_TRY(W.rc.alloc((size_t)nc * ((h->nrep > 1 || h->mixed_cg()) ? kChunk : 1)), "alloc");
  NMG_CUDA_TRY(cudaMemcpy(W.ainv.p, Ainv.data(), sizeof(double) * nc * nc, cudaMemcpyHostToDevice), "h2d");
  {
    std::vector<float> a32(Ainv.begin(), Ainv.end());
    NMG_CUDA_TRY(W.ainv32.alloc((size_t)nc * nc), "alloc coarse inverse (FP32)");
    NMG_CUDA_TRY(W.rc32.alloc((size_t)nc * kChunk), "alloc");
    NMG_CUDA_TRY(W.rw32.alloc((size_t)nc * kChunk), "alloc");
    NMG_CUDA_TRY(cudaMemcpy(W.ainv32.p, a32.data(), sizeof(float) * nc * nc, cudaMemcpyHostToDevice), "h2d");
  }
  W.nc = nc;
  return 0;
}

// Orders h->stream after the last warm-start factor formed for basis slot
// ev_slot on the auxiliary stream: that kernel reads the basis (its ring,
// Gram matrix) which the next solve or reset of the slot overwrites.
void wait_basis_factor(nmg_handle *h, int ev_slot) {
  const Workspace &W = h->ws;
  if (W.aux && ev_slot >= 0 && ev_slot < (int)W.ev_ldl.size())
    cudaStreamWaitEvent(h->stream, W.ev_ldl[ev_slot], 0);
}

int run_cg(nmg_handle *h, int mode, const double *b, double *x, double rtol, double atol, int maxits) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  CGArgs a;
  a.N = M.N; a.mode = mode & 1;   // slots 2 and 3: the same operators, separate warm-start bases
  a.row_ptr = M.row_ptr; a.col_idx = M.col_idx; a.b_of_node = M.b_of_node; a.K = M.K;
  a.dinv = (mode & 1) == 0 ? W.dinv_n.p : W.dinv_d.p;
  a.b = b; a.x = x; a.r = W.cg_r; a.z = W.cg_z; a.p = W.cg_p; a.q = W.cg_q; a.red = W.red;
  a.w = W.cg_w; a.flags = W.bar; a.tot = W.cg_tot;
  a.bar = W.bar; a.err = W.err; a.iters = W.iters;
  a.rtol = rtol; a.atol = atol; a.maxits = maxits;
  a.perm = W.perm; a.prow = W.prow; a.pcol = W.pcol; a.pbnd = W.pbnd; a.pK = W.pK; a.xperm = W.xperm;
  a.coarse = ((mode & 1) == 0 && W.nc > 0) ? 1 : 0;
  a.nc = W.nc; a.ainv = W.ainv; a.rc = W.rc;
  // fresh barrier words per solve: epochs restart at 1 inside the kernel
  cudaMemsetAsync(W.bar.p, 0, sizeof(unsigned) * (W.cg_blocks + 1), h->stream);
  wait_basis_factor(h, mode);
  NMG_PROF_BEGIN(h, 1 + (mode & 1));
  cudaError_t e;
  {
    int cap = W.cg_nnz_cap;
    CGBasis basis;
    basis.b = W.basis_b.p + (size_t)mode * kBasis * M.N;
    basis.x = W.basis_x.p + (size_t)mode * kBasis * M.N;
    basis.gram = W.basis_gram.p + mode * kBasis * kBasis;
    basis.ring = W.basis_ring.p + 2 * mode;
    void *args3[] = {&a, &cap, &basis};
    e = cudaLaunchCooperativeKernel((const void *)k_cg3, dim3(W.cg_blocks), dim3(kCGThreads), args3,
                                    (size_t)W.cg_smem_bytes, h->stream);
  }
  NMG_PROF_END(h);
  ++h->launches;
  if (e != cudaSuccess) {
    h->last_error = std::string("CG launch failed: ") + cudaGetErrorString(e);
    return 100;
  }
  return 0;
}

// Ensemble CG: nm <= kChunk right-hand sides (member m at b + m * N).
// bslot: warm-start basis slot of a single simulation (-1: `mode`); mp: 1
// mixed precision, 0 FP64, -1 the handle's forward choice.
int run_cgm(nmg_handle *h, int mode, int c0, const double *b, double *x, int nm, double rtol, double atol,
            int maxits, int bslot = -1, int mp_sel = -1) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  CGArgs a;
  a.N = M.N; a.mode = mode;
  a.row_ptr = M.row_ptr; a.col_idx = M.col_idx; a.b_of_node = M.b_of_node; a.K = M.K;
  a.dinv = mode == 0 ? W.dinv_n.p : W.dinv_d.p;
  a.b = b; a.x = x; a.r = W.cg_r; a.z = W.cg_z; a.p = W.cg_p; a.q = W.cg_q; a.red = W.red;
  a.w = W.cg_w; a.flags = W.bar; a.tot = W.cg_tot;
  a.bar = W.bar; a.err = W.err; a.iters = W.iters;
  a.rtol = rtol; a.atol = atol; a.maxits = maxits;
  a.perm = W.perm; a.prow = W.prow; a.pcol = W.pcol; a.pbnd = W.pbnd; a.pK = W.pK; a.xperm = W.xperm;
  a.coarse = (mode == 0 && W.nc > 0) ? 1 : 0;
  a.nc = W.nc; a.ainv = W.ainv; a.rc = W.rc;
  a.ainv32 = W.ainv32; a.rc32 = W.rc32; a.z32 = W.z32; a.rw32 = W.rw32;
  a.mcol = W.mcol; a.mmid = W.mmid; a.mK0 = W.mK; a.mK1 = W.mK.p ? W.mK.p + M.nnz : nullptr;
  a.mK32_0 = W.mK32; a.mK32_1 = W.mK32.p ? W.mK32.p + M.nnz : nullptr;
  a.eta = 1e-3f; a.max_outer = 10;
  a.local_sweeps = h->opt.cg_local_sweeps > 1 ? h->opt.cg_local_sweeps : 1;
  cudaMemsetAsync(W.bar.p, 0, sizeof(unsigned) * (W.cg_blocks + 1), h->stream);
  int cap = W.cg_nnz_cap;
  CGBasis basis;
  int ev_slot;   // the basis slot's event
  if (h->nrep > 1) {
    const size_t slot = (size_t)mode * h->nrep + c0;   // first member of this chunk
    basis.b = W.ens_basis_b.p + slot * kBasis * M.N;
    basis.x = W.ens_basis_x.p + slot * kBasis * M.N;
    basis.gram = W.ens_basis_gram.p + slot * kBasis * kBasis;
    basis.ring = W.ens_basis_ring.p + 2 * slot;
    basis.ldl = W.ens_basis_ldl.p ? W.ens_basis_ldl.p + slot : nullptr;
    ev_slot = kCGSlots + (int)slot;
  } else {   // one simulation: the single-solve bases of slot bslot (default `mode`)
    const int sl = bslot >= 0 ? bslot : mode;
    basis.b = W.basis_b.p + (size_t)sl * kBasis * M.N;
    basis.x = W.basis_x.p + (size_t)sl * kBasis * M.N;
    basis.gram = W.basis_gram.p + sl * kBasis * kBasis;
    basis.ring = W.basis_ring.p + 2 * sl;
    basis.ldl = W.basis_ldl.p ? W.basis_ldl.p + sl : nullptr;
    ev_slot = sl;
  }
  const bool mp_f = (mp_sel >= 0 ? mp_sel == 1 : h->opt.cg_precision == 1) && W.aux && basis.ldl &&
                    ev_slot < (int)W.ev_ldl.size();
  if (!mp_f) basis.ldl = nullptr;   // the kernel factors in place
  wait_basis_factor(h, ev_slot);   // this basis's last factor is formed
  void *args[] = {&a, &cap, &nm, &basis};
  const bool mp = mp_sel >= 0 ? mp_sel == 1 : h->opt.cg_precision == 1;
  const void *fn;
  if (mp) fn = nm <= 2 ? (const void *)k_cgm_mp<2> : (nm <= 4 ? (const void *)k_cgm_mp<4> : (const void *)k_cgm_mp<8>);
  else fn = nm <= 2 ? (const void *)k_cgm<2> : (nm <= 4 ? (const void *)k_cgm<4> : (const void *)k_cgm<8>);
  NMG_PROF_BEGIN(h, 1 + mode);
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(W.cg_blocks), dim3(kCGThreads), args,
                                              (size_t)(mp ? W.cg_smem_mp : W.cg_smem_bytes), h->stream);
  NMG_PROF_END(h);
  ++h->launches;
  if (e != cudaSuccess) {
    h->last_error = std::string("ensemble CG launch failed: ") + cudaGetErrorString(e);
    return 100;
  }
  if (mp_f) {   // the next solve's warm-start factor, off the main stream
    cudaEventRecord(W.ev_cg, h->stream);
    cudaStreamWaitEvent(W.aux, W.ev_cg, 0);
    k_gram_factor<<<1, 32 * kChunk, 0, W.aux>>>(basis, nm);
    ++h->launches;
    cudaEventRecord(W.ev_ldl[ev_slot], W.aux);
    if (cudaGetLastError() != cudaSuccess) {
      h->last_error = "mixed-precision CG: the warm-start factor could not be launched";
      return 100;
    }
  }
  return 0;
}

}  // namespace

int cg_solve(nmg_handle *h, int slot, const double *b, double *x, double rtol, double atol, int maxits) {
  if (slot >= 2 && h->opt.adjoint_cg_precision == 1)   // the adjoint's solves, mixed precision
    return run_cgm(h, slot & 1, 0, b, x, 1, rtol, atol, maxits, slot, 1);
  return run_cg(h, slot, b, x, rtol, atol, maxits);
}

void cg_reset_basis(nmg_handle *h, int slot) {
  wait_basis_factor(h, slot);
  cudaMemsetAsync(h->ws.basis_ring.p + 2 * slot, 0, sizeof(int) * 2, h->stream);
}

int init_workspace(nmg_handle *h, std::string &err) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const int N = M.N, nb = M.nb;
  const int B = h->nrep, BC = std::min(B, kChunk);   // members; members per CG / BEM launch
  const size_t n3 = 3 * (size_t)N * B, nB = (size_t)N * B;
  for (DevBuf<double> *b : {&W.m, &W.h_ext, &W.h_exch, &W.h_demag, &W.h_anis, &W.h_total, &W.dmdt})
    NMG_CUDA_TRY(b->alloc(n3), "alloc field");
  for (DevBuf<double> *b : {&W.rho, &W.phi1, &W.phi2, &W.phi, &W.rhs2})
    NMG_CUDA_TRY(b->alloc(nB), "alloc scalar field");
  const int BCv = B > 1 ? kChunk : 1;   // ensemble CG vectors are member-minor with stride up to kChunk
  for (DevBuf<double> *b : {&W.cg_r, &W.cg_z, &W.cg_p, &W.cg_q})
    NMG_CUDA_TRY(b->alloc((size_t)N * BCv), "alloc CG vectors");
  for (DevBuf<double> *b : {&W.dinv_n, &W.dinv_d})
    NMG_CUDA_TRY(b->alloc(N), "alloc scalar field");
  NMG_CUDA_TRY(W.b1.alloc(nb > 0 ? (size_t)nb * B : 1), "alloc");
  NMG_CUDA_TRY(W.b2.alloc(nb > 0 ? (size_t)nb * B : 1), "alloc");
  NMG_CUDA_TRY(W.E5.alloc(5 * nB), "alloc");
  cudaMemsetAsync(W.m.p, 0, sizeof(double) * n3, h->stream);
  cudaMemsetAsync(W.h_ext.p, 0, sizeof(double) * n3, h->stream);
  cudaMemsetAsync(W.phi1.p, 0, sizeof(double) * nB, h->stream);
  cudaMemsetAsync(W.phi2.p, 0, sizeof(double) * nB, h->stream);
  cudaMemsetAsync(W.phi.p, 0, sizeof(double) * nB, h->stream);
  for (DevBuf<double> *b : {&W.h_exch, &W.h_demag, &W.h_anis, &W.h_total, &W.dmdt})
    cudaMemsetAsync(b->p, 0, sizeof(double) * n3, h->stream);
  // CG grid: one row per thread when it fits in one co-resident wave.
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg3, kCGThreads, 0);
  int max_blocks = per_sm * h->sm_count;
  int want = nblk(N, kCGThreads);
  W.cg_blocks = want < max_blocks ? want : max_blocks;
  if (W.cg_blocks < 1) W.cg_blocks = 1;
  // Shared-memory CG: one row per thread, each block's CSR rows resident.
  {
    int rc_order = build_cg_ordering(h, err);
    if (rc_order) return rc_order;
    std::vector<int32_t> rp(N + 1);
    NMG_CUDA_TRY(cudaMemcpy(rp.data(), W.prow.p, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost), "d2h");
    int cap = 0;
    for (int r0 = 0; r0 < N; r0 += kCGThreads) {
      int r1 = r0 + kCGThreads < N ? r0 + kCGThreads : N;
      cap = rp[r1] - rp[r0] > cap ? rp[r1] - rp[r0] : cap;
    }
    cap = (cap + 1) & ~1;
    const int bytes = cap * (int)(sizeof(double) + sizeof(int));
    W.cg_smem_bytes = 0;
    W.cg_nnz_cap = cap;
    // The attribute is per function (shared by every handle): always raise it
    // to the cap so that handles with different meshes do not undercut it.
    if (bytes <= 160 * 1024 &&
        cudaFuncSetAttribute(k_cg3, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024) == cudaSuccess) {
      int per3 = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per3, k_cg3, kCGThreads, bytes);
      if (per3 > 0 && want <= per3 * h->sm_count) {
        W.cg_smem_bytes = bytes;
        W.cg_blocks = want;
      }
    }
    cudaGetLastError();
    if (W.cg_smem_bytes == 0 && h->opt.do_demag) {
      err = "mesh too large for the resident CG (one node per thread in one co-resident wave: at most " +
            std::to_string(per_sm * h->sm_count * kCGThreads) + " nodes here)";
      return 4;
    }
    // CSR (FP64 + FP32 values, columns), the block's u, and with the coarse
    // level the whole coarse residual and its direction term plus this
    // block's rows of the coarse inverse (FP32)
    W.cg_smem_mp = cap * (int)(sizeof(double) + sizeof(int) + sizeof(float)) +
                   (int)sizeof(float) * (kCGThreads * kChunk + (W.nc > 0 ? 2 * W.nc * kChunk + (kCGThreads / kAgg) * W.nc : 0));
    const bool mp = h->mixed_cg();
    if ((B > 1 || mp) && h->opt.do_demag) {
      // the ensemble / mixed-precision CG kernels: up to kChunk members per row
      if (mp && W.nc * kChunk > kRwPer * 4 * kCGThreads) {
        err = "mesh too large for the mixed-precision CG (" + std::to_string(W.nc) + " aggregates, at most " +
              std::to_string(kRwPer * 4 * kCGThreads / kChunk) + ")";
        return 4;
      }
      struct Need { const void *fn; int smem; };
      std::vector<Need> needs;
      if (mp)   // forward mixed CG, or the adjoint's
        for (const void *fn : {(const void *)k_cgm_mp<2>, (const void *)k_cgm_mp<4>, (const void *)k_cgm_mp<8>})
          needs.push_back({fn, W.cg_smem_mp});
      if (B > 1 && h->opt.cg_precision != 1)   // FP64 ensemble CG
        for (const void *fn : {(const void *)k_cgm<2>, (const void *)k_cgm<4>, (const void *)k_cgm<8>})
          needs.push_back({fn, W.cg_smem_bytes});
      for (const Need &nd : needs) {
        int per = 0;
        if (nd.smem > 160 * 1024 ||
            cudaFuncSetAttribute(nd.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, nd.fn, kCGThreads, nd.smem) != cudaSuccess ||
            per * h->sm_count < W.cg_blocks) {
          cudaGetLastError();
          err = "mesh too large for the ensemble CG (" + std::to_string(W.cg_blocks) + " co-resident blocks needed)";
          return 4;
        }
      }
    }
  }
  // BEM product grid: every resident warp streams an equal share of the
  // flattened matrix (units of 32 bytes; rows of ld entries).
  size_t part_n = 1;
  M.ld = (nb + 7) / 8 * 8;   // row stride of the BEM matrix (fill_bem stores with it)
  if (nb > 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemv_f64, kGemvThreads, 0);
    int per_sm32 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm32, k_gemv_f32, kGemvThreads, 0);
    per_sm = std::max(1, std::min(std::min(per_sm, per_sm32), 8));
    W.gemv_blocks = per_sm * h->sm_count;
    const long long warps = (long long)W.gemv_blocks * (kGemvThreads / 32);
    for (int f = 0; f < 2; ++f) {
      const long long Q = M.ld / (f == 0 ? 4 : 8), total = (long long)nb * Q;
      const long long seg = std::max<long long>(1, (total + warps - 1) / warps);
      W.gemv_seg[f] = seg;
      W.gemv_maxr[f] = (int)((seg + Q - 1) / Q + 1);
      part_n = std::max(part_n, (size_t)(warps * W.gemv_maxr[f]));
    }
  }
  // partials (kChunk members for the ensemble), then FP32 copies of x padded to ld
  part_n *= (B > 1 ? kChunk : 1);
  if (B > 1 && nb > 0)   // FP32 / compensated tiles: one partial per (slab, row, member)
    part_n = std::max(part_n, (size_t)((M.ld + std::min(kRegSlab, kDfCols) - 1) / std::min(kRegSlab, kDfCols)) *
                                  nb * kChunk);
  W.gemv_x32_off = (part_n + 7) / 8 * 8;
  // FP32 x copies: BC members, or BC (xh, xl) pairs for the compensated product
  NMG_CUDA_TRY(W.bpart.alloc(W.gemv_x32_off + (size_t)BC * M.ld + 8), "alloc gemv partials");
  // anchored ensemble product in the FP16 fragment form (the matrix copy is
  // packed by fill_bem): warps stream equal shares of the KT x KT tiles
  if (nb > 0 && B > 1 && h->opt.bem_precision == 2 && h->opt.bem_anchor_tol > 0.0 && h->opt.anchor_product == 1) {
    M.h16_kt = (nb + 15) / 16;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_h16mma, 256, 0);
    W.h16_blocks = std::max(1, std::min(per_sm, 8)) * h->sm_count;
    const long long nwarps = (long long)W.h16_blocks * 8, TT = (long long)M.h16_kt * M.h16_kt;
    W.h16_seg = std::max<long long>(1, (TT + nwarps - 1) / nwarps);
    W.h16_maxr = (int)((W.h16_seg + M.h16_kt - 1) / M.h16_kt + 1);
    NMG_CUDA_TRY(W.x16f.alloc((size_t)M.h16_kt * 32 * 4), "alloc FP16 x fragments");
    NMG_CUDA_TRY(W.x16scale.alloc(kChunk), "alloc");
    NMG_CUDA_TRY(W.h16part.alloc((size_t)nwarps * W.h16_maxr * 128), "alloc FP16 product partials");
  }
  // 2 parities x kCG2MaxRed values per block (at least 1024 blocks: averages use it too)
  size_t red_n = 2 * (size_t)kCG2MaxRed * (size_t)(W.cg_blocks > 1024 ? W.cg_blocks : 1024);
  NMG_CUDA_TRY(W.red.alloc(red_n), "alloc reductions");
  NMG_CUDA_TRY(W.bar.alloc(W.cg_blocks + 2), "alloc barrier");
  NMG_CUDA_TRY(W.cg_w.alloc((size_t)N * BC), "alloc");
  NMG_CUDA_TRY(W.basis_b.alloc(kCGSlots * (size_t)kBasis * N), "alloc CG basis");
  NMG_CUDA_TRY(W.basis_x.alloc(kCGSlots * (size_t)kBasis * N), "alloc CG basis");
  NMG_CUDA_TRY(W.basis_gram.alloc(kCGSlots * kBasis * kBasis), "alloc");
  if (h->mixed_cg() && h->opt.do_demag) {   // the mixed-precision CG's warm-start factors
    NMG_CUDA_TRY(W.basis_ldl.alloc(kCGSlots), "alloc");
    NMG_CUDA_TRY(cudaMemset(W.basis_ldl.p, 0, sizeof(GramLDL) * kCGSlots), "memset");
    NMG_CUDA_TRY(cudaStreamCreateWithFlags(&W.aux, cudaStreamNonBlocking), "auxiliary stream");
    NMG_CUDA_TRY(cudaEventCreateWithFlags(&W.ev_cg, cudaEventDisableTiming), "event");
    W.ev_ldl.assign(kCGSlots + 2 * (size_t)B, nullptr);
    for (cudaEvent_t &ev : W.ev_ldl) NMG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
  }
  NMG_CUDA_TRY(W.basis_ring.alloc(2 * kCGSlots), "alloc");
  if (B > 1) {
    NMG_CUDA_TRY(W.ens_basis_b.alloc(2 * (size_t)B * kBasis * N), "alloc ensemble CG basis");
    NMG_CUDA_TRY(W.ens_basis_x.alloc(2 * (size_t)B * kBasis * N), "alloc ensemble CG basis");
    NMG_CUDA_TRY(W.ens_basis_gram.alloc(2 * (size_t)B * kBasis * kBasis), "alloc");
    if (h->mixed_cg() && h->opt.do_demag) {
      NMG_CUDA_TRY(W.ens_basis_ldl.alloc(2 * (size_t)B), "alloc");
      NMG_CUDA_TRY(cudaMemset(W.ens_basis_ldl.p, 0, sizeof(GramLDL) * 2 * B), "memset");
    }
    NMG_CUDA_TRY(W.ens_basis_ring.alloc(4 * (size_t)B), "alloc");
    cudaMemsetAsync(W.ens_basis_ring.p, 0, sizeof(int) * 4 * B, h->stream);
  }
  cudaMemsetAsync(W.basis_ring.p, 0, sizeof(int) * 2 * kCGSlots, h->stream);
  NMG_CUDA_TRY(W.cg_tot.alloc(2 * 4), "alloc");
  if (h->opt.bem_anchor_tol > 0.0 && h->opt.bem_precision == 2 && nb > 0) {
    const int nchunk = (B + kChunk - 1) / kChunk;
    NMG_CUDA_TRY(W.anc_x.alloc((size_t)nb * B), "alloc BEM anchor");
    NMG_CUDA_TRY(W.anc_y.alloc((size_t)nb * B), "alloc BEM anchor");
    NMG_CUDA_TRY(W.anc_mx.alloc(2 * kChunk), "alloc");
    NMG_CUDA_TRY(W.anc_flag.alloc(2 * (size_t)nchunk), "alloc");
    NMG_CUDA_TRY(W.anc_count.alloc(2), "alloc");
    cudaMemsetAsync(W.anc_mx.p, 0, sizeof(unsigned long long) * 2 * kChunk, h->stream);
    cudaMemsetAsync(W.anc_flag.p, 0, sizeof(int) * 2 * nchunk, h->stream);
    cudaMemsetAsync(W.anc_count.p, 0, sizeof(long long) * 2, h->stream);
  }
  NMG_CUDA_TRY(W.iters.alloc(4), "alloc");
  cudaMemsetAsync(W.bar.p, 0, sizeof(unsigned) * 2, h->stream);
  cudaMemsetAsync(W.iters.p, 0, sizeof(int) * 4, h->stream);
  k_dinv<<<nblk(N, 256), 256, 0, h->stream>>>(N, M.diag_pos, M.K, M.b_of_node, W.dinv_n, W.dinv_d); ++h->launches;
  NMG_CUDA_TRY(cudaGetLastError(), "workspace init");
  NMG_CUDA_TRY(cudaStreamSynchronize(h->stream), "workspace init");
  return 0;
}

void bem_gemv(nmg_handle *h, const double *x, double *y) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const int nb = M.nb;
  if (h->opt.bem_precision == 3) {   // tensor cores, split BF16
    if (bem_tc(h, x, y, 1)) h->tc.failed = 1;   // reported by rhs_eval
    return;
  }
  const int f = (h->opt.bem_precision >= 1 && M.bem32.p) ? 1 : 0;
  const long long seg = W.gemv_seg[f];
  const int maxr = W.gemv_maxr[f];
  if (h->anchored() && W.anc_x.p) {   // anchored compensated product (one simulation)
    float *xh = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
    float *xl = xh + M.ld;
    int *flag = W.anc_flag.p, *valid = W.anc_flag.p + 1;
    k_anchor_drift<<<nblk(M.ld, 256), 256, 0, h->stream>>>(nb, M.ld, 1, x, W.anc_x, xh, W.anc_mx); ++h->launches;
    k_anchor_decide<<<1, 32, 0, h->stream>>>(1, h->opt.bem_anchor_tol, W.anc_mx, valid, flag, W.anc_count);
    ++h->launches;
    k_split_x<<<nblk(M.ld, 256), 256, 0, h->stream>>>(nb, M.ld, 1, x, xh, xl, flag); ++h->launches;
    {
      NMG_PROF_BEGIN(h, 0);
      k_gemv_df<<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, M.bem32, M.bem16lo, xh, xl,
                                                               W.bpart, flag);
      ++h->launches;
      NMG_PROF_END(h);
    }
    {
      NMG_PROF_BEGIN(h, 5);
      k_gemv_f32<<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, M.bem32, xh, W.bpart, flag);
      ++h->launches;
      NMG_PROF_END(h);
    }
    k_anchor_row_sum<<<nblk(nb, 256), 256, 0, h->stream>>>(nb, (long long)(M.ld / 8), seg, maxr,
                                                           (long long)W.gemv_blocks * (kGemvThreads / 32), W.bpart,
                                                           flag, valid, x, W.anc_x, W.anc_y, y);
    ++h->launches;
    return;
  }
  if (f == 1 && M.bem16lo.p && !h->bem_fp32_only) {   // compensated FP32 pair product
    float *xh = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
    float *xl = xh + M.ld;
    k_split_x<<<nblk(M.ld, 256), 256, 0, h->stream>>>(nb, M.ld, 1, x, xh, xl); ++h->launches;
    NMG_PROF_BEGIN(h, 0);
    k_gemv_df<<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, M.bem32, M.bem16lo, xh, xl, W.bpart);
    ++h->launches;
    NMG_PROF_END(h);
  } else if (f == 1) {
    float *x32 = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
    k_to_f32_vec<<<nblk(M.ld, 256), 256, 0, h->stream>>>(nb, M.ld, x, x32); ++h->launches;
    NMG_PROF_BEGIN(h, 0);
    k_gemv_f32<<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, M.bem32, x32, W.bpart); ++h->launches;
    NMG_PROF_END(h);
  } else {
    NMG_PROF_BEGIN(h, 0);
    k_gemv_f64<<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, M.bem, x, W.bpart); ++h->launches;
    NMG_PROF_END(h);
  }
  k_row_sum<<<nblk(nb, 256), 256, 0, h->stream>>>(nb, (long long)(M.ld / (f == 0 ? 4 : 8)), seg, maxr,
                                                  (long long)W.gemv_blocks * (kGemvThreads / 32), W.bpart, y);
  ++h->launches;
}

// Y = B X for the ensemble (member m at x + m * nb), kChunk members per pass.
void bem_gemm(nmg_handle *h, const double *x, double *y) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const int nb = M.nb, B = h->nrep;
  if (h->opt.bem_precision == 3) {   // every member in one tensor-core product
    if (bem_tc(h, x, y, B)) h->tc.failed = 1;   // reported by rhs_eval
    return;
  }
  const int f = (h->opt.bem_precision >= 1 && M.bem32.p) ? 1 : 0;
  const long long seg = W.gemv_seg[f];
  const int maxr = W.gemv_maxr[f];
  const long long Q = M.ld / (f == 0 ? 4 : 8);
  const long long nwarps = (long long)W.gemv_blocks * (kGemvThreads / 32);
  for (int c0 = 0; c0 < B; c0 += kChunk) {
    const int nm = std::min(kChunk, B - c0);
    const int MB = nm <= 2 ? 2 : (nm <= 4 ? 4 : 8);
    const double *xc = x + (size_t)c0 * nb;
    if (h->anchored() && W.anc_x.p) {   // anchored compensated product for this chunk
      float *xh = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
      float *xl = xh + (size_t)nm * M.ld;
      int *flag = W.anc_flag.p + 2 * (c0 / kChunk), *valid = flag + 1;
      double *ax = W.anc_x.p + (size_t)c0 * nb, *ay = W.anc_y.p + (size_t)c0 * nb;
      k_anchor_drift<<<nblk((long long)M.ld * nm, 256), 256, 0, h->stream>>>(nb, M.ld, nm, xc, ax, xh, W.anc_mx);
      ++h->launches;
      const bool h16 = M.bem16f.p && W.h16part.p;   // FP16 fragment difference product
      k_anchor_decide<<<1, 32, 0, h->stream>>>(nm, h->opt.bem_anchor_tol, W.anc_mx, valid, flag, W.anc_count,
                                               h16 ? W.x16scale.p : nullptr);
      ++h->launches;
      k_split_x<<<nblk((long long)M.ld * nm, 256), 256, 0, h->stream>>>(nb, M.ld, nm, xc, xh, xl, flag);
      ++h->launches;
      const int nslab_df = (M.ld + kDfCols - 1) / kDfCols, nslab_32 = (M.ld + kRegSlab - 1) / kRegSlab;
      {
        dim3 grid(nslab_df, (nb + kDfRows - 1) / kDfRows);
        NMG_PROF_BEGIN(h, 0);
        if (MB == 2) k_gemm_df<2><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart, flag);
        else if (MB == 4) k_gemm_df<4><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart, flag);
        else k_gemm_df<8><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart, flag);
        NMG_PROF_END(h);
        ++h->launches;
      }
      if (h16) {
        const int KT = M.h16_kt;
        const long long nwarps = (long long)W.h16_blocks * 8;
        uint2 *x16 = reinterpret_cast<uint2 *>(W.x16f.p);
        k_pack_x16f<<<nblk((long long)KT * 32, 256), 256, 0, h->stream>>>(nb, M.ld, nm, KT, xh, W.x16scale, x16, flag);
        ++h->launches;
        {
          NMG_PROF_BEGIN(h, 5);
          k_gemm_h16mma<<<W.h16_blocks, 256, 0, h->stream>>>((long long)KT * KT, KT, W.h16_seg, W.h16_maxr,
                                                            reinterpret_cast<const uint4 *>(M.bem16f.p), x16,
                                                            reinterpret_cast<float4 *>(W.h16part.p), flag);
          NMG_PROF_END(h);
          ++h->launches;
        }
        k_anchor_h16_sum<<<nblk((long long)nb * nm, 256), 256, 0, h->stream>>>(
            nb, nslab_df, nm, MB, W.bpart, W.h16part, KT, W.h16_seg, W.h16_maxr, nwarps, 1.0 / (double)M.h16_scale,
            W.x16scale, flag, valid, xc, ax, ay, y + (size_t)c0 * nb);
        ++h->launches;
        continue;
      }
      {
        dim3 grid(nslab_32, (nb + kRegRows - 1) / kRegRows);
        NMG_PROF_BEGIN(h, 5);
        if (MB == 2) k_gemm_f32r<2><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, xh, W.bpart, flag);
        else if (MB == 4) k_gemm_f32r<4><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, xh, W.bpart, flag);
        else k_gemm_f32r<8><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, xh, W.bpart, flag);
        NMG_PROF_END(h);
        ++h->launches;
      }
      k_anchor_slab_sum<<<nblk((long long)nb * nm, 256), 256, 0, h->stream>>>(
          nb, nslab_df, nslab_32, nm, MB, W.bpart, flag, valid, xc, ax, ay, y + (size_t)c0 * nb);
      ++h->launches;
      continue;
    }
    if (f == 1 && M.bem16lo.p && !h->bem_fp32_only) {   // compensated FP32 pair product on tiles
      float *xh = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
      float *xl = xh + (size_t)nm * M.ld;
      k_split_x<<<nblk((long long)M.ld * nm, 256), 256, 0, h->stream>>>(nb, M.ld, nm, xc, xh, xl); ++h->launches;
      const int nslab = (M.ld + kDfCols - 1) / kDfCols;
      dim3 grid(nslab, (nb + kDfRows - 1) / kDfRows);
      NMG_PROF_BEGIN(h, 0);
      if (MB == 2) k_gemm_df<2><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart);
      else if (MB == 4) k_gemm_df<4><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart);
      else k_gemm_df<8><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, M.bem16lo, xh, xl, W.bpart);
      NMG_PROF_END(h);
      ++h->launches;
      k_slab_sum_m<<<nblk((long long)nb * nm, 256), 256, 0, h->stream>>>(nb, nslab, nm, MB, W.bpart,
                                                                         y + (size_t)c0 * nb);
      ++h->launches;
      continue;
    }
    if (f == 1) {
      float *x32 = reinterpret_cast<float *>(W.bpart.p + W.gemv_x32_off);
      k_to_f32_vec<<<nblk((long long)M.ld * nm, 256), 256, 0, h->stream>>>(nb, M.ld, xc, x32, nm); ++h->launches;
      const int nslab = (M.ld + kRegSlab - 1) / kRegSlab;
      dim3 grid(nslab, (nb + kRegRows - 1) / kRegRows);
      NMG_PROF_BEGIN(h, 0);
      if (MB == 2) k_gemm_f32r<2><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, x32, W.bpart);
      else if (MB == 4) k_gemm_f32r<4><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, x32, W.bpart);
      else k_gemm_f32r<8><<<grid, 256, 0, h->stream>>>(nb, M.ld, nm, M.bem32, x32, W.bpart);
      NMG_PROF_END(h);
      ++h->launches;
      k_slab_sum_m<<<nblk((long long)nb * nm, 256), 256, 0, h->stream>>>(nb, nslab, nm, MB, W.bpart,
                                                                         y + (size_t)c0 * nb);
      ++h->launches;
      continue;
    } else {
      NMG_PROF_BEGIN(h, 0);
      if (MB == 2) k_gemm_f64<2><<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, nm, M.bem, xc, W.bpart);
      else if (MB == 4) k_gemm_f64<4><<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, nm, M.bem, xc, W.bpart);
      else k_gemm_f64<8><<<W.gemv_blocks, kGemvThreads, 0, h->stream>>>(nb, M.ld, seg, maxr, nm, M.bem, xc, W.bpart);
      NMG_PROF_END(h);
    }
    ++h->launches;
    k_row_sum_m<<<nblk((long long)nb * nm, 256), 256, 0, h->stream>>>(nb, Q, seg, maxr, nwarps, nm, MB, W.bpart,
                                                                      y + (size_t)c0 * nb);
    ++h->launches;
  }
}

int check_device_error(nmg_handle *h, const char *where) {
  if (h->pot) {   // several materials: the potential mesh's solves flag their errors there
    const int rc = check_device_error(h->pot, where);
    if (rc) {
      h->last_error = h->pot->last_error;
      return rc;
    }
  }
  int derr = 0;
  cudaError_t e = cudaMemcpyAsync(&derr, h->ws.err.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    h->last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return 100;
  }
  if (derr) {
    cudaMemsetAsync(h->ws.err.p, 0, sizeof(int), h->stream);
    if (derr & ERR_BARRIER) h->last_error = std::string(where) + ": grid barrier timed out";
    else if (derr & ERR_NONFINITE) h->last_error = std::string(where) + ": solver produced non-finite values";
    else if (derr & ERR_CG_MAXITS) h->last_error = std::string(where) + ": CG reached its iteration limit";
    else h->last_error = std::string(where) + ": device error flag " + std::to_string(derr);
    return (derr & ERR_BARRIER) ? 7 : ((derr & ERR_NONFINITE) ? 6 : 5);
  }
  return 0;
}

// The demag pipeline from the charges in W.rho (all members) to the
// potential W.phi: Neumann solve, boundary gather, BEM product, Dirichlet
// load and solve, phi = phi1 + phi2 (nmag_lam.py:740-760).
int demag_from_rho(nmg_handle *h) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  cudaStream_t s = h->stream;
  const int N = M.N;
  const int B = h->nrep;
  if (B > 1) {
    // ensemble: the same pipeline over B members, kChunk members per CG / BEM launch
    const long long NB = (long long)N * B;
    for (int c0 = 0; c0 < B; c0 += kChunk)
      if (run_cgm(h, 0, c0, W.rho.p + (size_t)c0 * N, W.phi1.p + (size_t)c0 * N, std::min(kChunk, B - c0),
                  h->opt.nbc_rtol, h->opt.nbc_atol, h->opt.nbc_maxits)) return 100;
    k_gather_b<<<nblk((long long)M.nb * B, 256), 256, 0, s>>>(M.nb, M.node_of_b, W.phi1, W.b1, N, B); ++h->launches;
    bem_gemm(h, W.b1, W.b2);
    k_dbc_rhs<<<nblk(NB, 256), 256, 0, s>>>(N, M.row_ptr, M.col_idx, M.K, M.b_of_node, W.b2, W.rhs2, W.phi2, M.nb, B);
    ++h->launches;
    for (int c0 = 0; c0 < B; c0 += kChunk)
      if (run_cgm(h, 1, c0, W.rhs2.p + (size_t)c0 * N, W.phi2.p + (size_t)c0 * N, std::min(kChunk, B - c0),
                  h->opt.dbc_rtol, h->opt.dbc_atol, h->opt.dbc_maxits)) return 100;
    k_add<<<nblk(NB, 256), 256, 0, s>>>((int)NB, W.phi1, W.phi2, W.phi); ++h->launches;
  } else {
    const bool mp = h->opt.cg_precision == 1;   // mixed-precision CG (one member)
    if (mp ? run_cgm(h, 0, 0, W.rho, W.phi1, 1, h->opt.nbc_rtol, h->opt.nbc_atol, h->opt.nbc_maxits)
           : run_cg(h, 0, W.rho, W.phi1, h->opt.nbc_rtol, h->opt.nbc_atol, h->opt.nbc_maxits)) return 100;
    k_gather_b<<<nblk(M.nb, 256), 256, 0, s>>>(M.nb, M.node_of_b, W.phi1, W.b1); ++h->launches;
    bem_gemv(h, W.b1, W.b2);
    k_dbc_rhs<<<nblk(N, 256), 256, 0, s>>>(N, M.row_ptr, M.col_idx, M.K, M.b_of_node, W.b2, W.rhs2, W.phi2); ++h->launches;
    if (mp ? run_cgm(h, 1, 0, W.rhs2, W.phi2, 1, h->opt.dbc_rtol, h->opt.dbc_atol, h->opt.dbc_maxits)
           : run_cg(h, 1, W.rhs2, W.phi2, h->opt.dbc_rtol, h->opt.dbc_atol, h->opt.dbc_maxits)) return 100;
    k_add<<<nblk(N, 256), 256, 0, s>>>(N, W.phi1, W.phi2, W.phi); ++h->launches;
  }
  return 0;
}

int rhs_eval(nmg_handle *h, const double *d_m, double *d_dmdt) {
  if (h->pot) return rhs_eval_sites(h, d_m, d_dmdt);   // several materials
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  cudaStream_t s = h->stream;
  const int N = M.N;
  const nmg_material &mt = h->mat;
  const int B = h->nrep;
  if (h->opt.do_demag && M.nb > 0) {
    k_div<<<nblk((long long)N * B, 256), 256, 0, s>>>(N, M.nnz, mt.Ms, M.row_ptr, M.col_idx,
                                                       h->ep.active ? h->ep.Dx.p : M.D.p, d_m, W.rho, B);
    ++h->launches;
    if (demag_from_rho(h)) return 100;
  }
  NodeArgs a;
  a.N = N; a.nnz = M.nnz; a.do_demag = (h->opt.do_demag && M.nb > 0) ? 1 : 0; a.nrep = B;
  a.row_ptr = M.row_ptr; a.col_idx = M.col_idx; a.K = h->exch_K(); a.G = M.G; a.ivol = M.ivol;
  a.m = d_m; a.phi = W.phi; a.h_ext = W.h_ext;
  a.anis_node = h->ep.active ? h->ep.anis.p : nullptr;
  a.anis_in = nullptr;
  if (h->ap.nh > 0) {
    k_anis_poly<<<nblk((long long)N * B, 128), 128, 0, s>>>((long long)N * B, d_m, h->ap.nh, h->ap.hpow, h->ap.hcoef,
                                                             W.h_anis); ++h->launches;
    a.anis_in = W.h_anis;
  }
  a.dmdc = nullptr;
  a.pin = h->pin.p;
  a.C4 = h->stt.c4; a.C5 = h->stt.c5;
  if (h->stt.on()) {
    k_stt_dmdc<<<nblk((long long)N * B, 128), 128, 0, s>>>(N, B, M.nnz, M.row_ptr, M.col_idx, M.G, M.ivol, d_m,
                                                            h->stt.j, h->stt.dmdc); ++h->launches;
    a.dmdc = h->stt.dmdc;
  }
  a.c_exch = mt.exch_coeff; a.C1 = mt.C1; a.C2 = mt.C2; a.C3 = mt.C3; a.K1 = mt.K1; a.anis = mt.anis_coeff;
  a.ax = mt.axis[0]; a.ay = mt.axis[1]; a.az = mt.axis[2];
  if (h->ep.active) { a.ax = h->ep.axis[0]; a.ay = h->ep.axis[1]; a.az = h->ep.axis[2]; }
  a.h_exch = W.h_exch; a.h_demag = W.h_demag; a.h_anis = W.h_anis; a.h_total = W.h_total;
  a.dmdt = d_dmdt ? d_dmdt : W.dmdt.p;
  {
    NMG_PROF_BEGIN(h, 3);
    k_heff_llg<<<nblk((long long)N * B, 128), 128, 0, s>>>(a); ++h->launches;
    NMG_PROF_END(h);
  }
  h->n_rhs++;
  if (h->tc.failed) {   // the tensor-core product could not be set up (message in last_error)
    h->tc.failed = 0;
    return 100;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

namespace {
// H_demag at the nodes from a potential: -(G_j phi)_i / vol_i (the demag
// term of k_heff_llg), 3 per node and member.
__global__ void k_neg_grad(int N, int nrep, int nnz, const int32_t *__restrict__ row_ptr,
                           const int32_t *__restrict__ col_idx, const double *__restrict__ G,
                           const double *__restrict__ ivol, const double *__restrict__ phi, double *__restrict__ out) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)N * nrep) return;
  const int b = (int)(g / N), i = (int)(g - (long long)b * N);
  const double *ph = phi + (size_t)b * N;
  double g0 = 0.0, g1 = 0.0, g2 = 0.0;
  for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
    const double pj = ph[col_idx[k]];
    g0 += G[k] * pj; g1 += G[(size_t)nnz + k] * pj; g2 += G[2 * (size_t)nnz + k] * pj;
  }
  const double iv = ivol[i];
  out[3 * (size_t)g] = -g0 * iv; out[3 * (size_t)g + 1] = -g1 * iv; out[3 * (size_t)g + 2] = -g2 * iv;
}

void swap_jac_buffers(Workspace &W, JacDemag &J) {
  W.rho.swap(J.rho); W.phi1.swap(J.phi1); W.phi2.swap(J.phi2); W.phi.swap(J.phi); W.rhs2.swap(J.rhs2);
  W.b1.swap(J.b1); W.b2.swap(J.b2);
  W.basis_b.swap(J.basis_b); W.basis_x.swap(J.basis_x); W.basis_gram.swap(J.basis_gram);
  W.basis_ldl.swap(J.basis_ldl); W.ens_basis_ldl.swap(J.ens_basis_ldl);
  W.basis_ring.swap(J.basis_ring);
  W.ens_basis_b.swap(J.ens_basis_b); W.ens_basis_x.swap(J.ens_basis_x); W.ens_basis_gram.swap(J.ens_basis_gram);
  W.ens_basis_ring.swap(J.ens_basis_ring);
  W.iters.swap(J.iters);
}

// J's buffers with the sizes of P's workspace, zeroed (empty bases, zero
// initial potentials).
int jac_alloc(nmg_handle *P, JacDemag &J) {
  Workspace &W = P->ws;
  std::pair<DevBuf<double> *, size_t> d[] = {
      {&J.rho, W.rho.n}, {&J.phi1, W.phi1.n}, {&J.phi2, W.phi2.n}, {&J.phi, W.phi.n}, {&J.rhs2, W.rhs2.n},
      {&J.b1, W.b1.n}, {&J.b2, W.b2.n}, {&J.basis_b, W.basis_b.n}, {&J.basis_x, W.basis_x.n},
      {&J.basis_gram, W.basis_gram.n}, {&J.ens_basis_b, W.ens_basis_b.n}, {&J.ens_basis_x, W.ens_basis_x.n},
      {&J.ens_basis_gram, W.ens_basis_gram.n}, {&J.hdv, 3 * (size_t)P->mesh.N * P->nrep}};
  for (auto &e : d) {
    if (e.first->alloc(e.second) != cudaSuccess) return 100;
    if (e.second) cudaMemsetAsync(e.first->p, 0, sizeof(double) * e.second, P->stream);
  }
  for (auto e : {std::make_pair(&J.basis_ldl, W.basis_ldl.n), std::make_pair(&J.ens_basis_ldl, W.ens_basis_ldl.n)}) {
    if (e.first->alloc(e.second) != cudaSuccess) return 100;
    if (e.second) cudaMemsetAsync(e.first->p, 0, sizeof(GramLDL) * e.second, P->stream);
  }
  std::pair<DevBuf<int> *, size_t> k[] = {
      {&J.basis_ring, W.basis_ring.n}, {&J.ens_basis_ring, W.ens_basis_ring.n}, {&J.iters, W.iters.n}};
  for (auto &e : k) {
    if (e.first->alloc(e.second) != cudaSuccess) return 100;
    if (e.second) cudaMemsetAsync(e.first->p, 0, sizeof(int) * e.second, P->stream);
  }
  J.ready = true;
  return 0;
}
}  // namespace

int jac_demag_solve(nmg_handle *P, JacDemag &J, double rtol) {
  Workspace &W = P->ws;
  const double nr = P->opt.nbc_rtol, dr = P->opt.dbc_rtol;
  swap_jac_buffers(W, J);
  // the direction is no small change of the anchored state, and the Newton
  // matrix needs no compensated product: the plain FP32 one where it exists
  P->anchor_hold++;
  P->bem_fp32_only++;
  P->opt.nbc_rtol = rtol;
  P->opt.dbc_rtol = rtol;
  const int rc = demag_from_rho(P);
  P->opt.nbc_rtol = nr;
  P->opt.dbc_rtol = dr;
  P->bem_fp32_only--;
  P->anchor_hold--;
  swap_jac_buffers(W, J);
  if (rc) return rc;
  const Mesh &M = P->mesh;
  k_neg_grad<<<nblk((long long)M.N * P->nrep, 256), 256, 0, P->stream>>>(M.N, P->nrep, M.nnz, M.row_ptr, M.col_idx,
                                                                          M.G, M.ivol, J.phi, J.hdv);
  ++P->launches;
  if (P->tc.failed) {
    P->tc.failed = 0;
    return 100;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

int demag_response(nmg_handle *h, const double *d_v) {
  if (h->pot) return demag_response_sites(h, d_v);
  Mesh &M = h->mesh;
  JacDemag &J = h->jd;
  if (!J.ready && jac_alloc(h, J)) {
    h->last_error = "exact Jacobian: cannot allocate the demag response buffers";
    return 100;
  }
  k_div<<<nblk((long long)M.N * h->nrep, 256), 256, 0, h->stream>>>(M.N, M.nnz, h->mat.Ms, M.row_ptr, M.col_idx,
                                                                     h->ep.active ? h->ep.Dx.p : M.D.p, d_v, J.rho,
                                                                     h->nrep);
  ++h->launches;
  return jac_demag_solve(h, J, h->jac_rtol);
}

int jac_prepare(nmg_handle *P, JacDemag &J) {
  if (J.ready) return 0;
  return jac_alloc(P, J);
}

int energy_density(nmg_handle *h, const double *d_m, double *d_E5) {
  if (h->pot) return energy_density_sites(h, d_m, d_E5);   // several materials
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const nmg_material &mt = h->mat;
  const int NB = M.N * h->nrep;   // pointwise over all members: E[k * NB + member * N + i]
  k_energy<<<nblk(NB, 256), 256, 0, h->stream>>>(NB, d_m, W.h_exch, W.h_demag, W.h_ext, mt.E_coeff_half,
                                                  mt.E_coeff_ext, mt.K1, mt.axis[0], mt.axis[1], mt.axis[2],
                                                  h->ap.ne, h->ap.epow, h->ap.ecoef, d_E5); ++h->launches;
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

int averages(nmg_handle *h, const double *d_m, double avg[3], double energies[5], int member) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  const int nblocks = 64;
  const double *E = energies ? W.E5.p + (size_t)member * M.N : nullptr;
  if (energies && energy_density(h, d_m, W.E5)) return 100;
  k_avg_partials<<<nblocks, 256, 0, h->stream>>>(M.N, d_m + (size_t)member * 3 * M.N, M.vol, E, W.red,
                                                 (size_t)M.N * h->nrep); ++h->launches;
  std::vector<double> part(9 * nblocks);
  if (cudaMemcpyAsync(part.data(), W.red.p, sizeof(double) * 9 * nblocks, cudaMemcpyDeviceToHost, h->stream) ||
      cudaStreamSynchronize(h->stream))
    return 100;
  double tot[9] = {0};
  for (int b = 0; b < nblocks; ++b)
    for (int j = 0; j < 9; ++j) tot[j] += part[9 * b + j];
  for (int d = 0; d < 3; ++d) avg[d] = tot[1 + d] / tot[0];
  if (energies) for (int k = 0; k < 5; ++k) energies[k] = tot[4 + k];
  return 0;
}

int max_dm(nmg_handle *h, const double *d_m, const double *d_mprev, double *out) {
  const int nblocks = 64;
  k_maxdm_partials<<<nblocks, 256, 0, h->stream>>>(h->mesh.N * h->nrep, d_m, d_mprev, h->ws.red); ++h->launches;
  double part[nblocks];
  if (cudaMemcpyAsync(part, h->ws.red.p, sizeof(double) * nblocks, cudaMemcpyDeviceToHost, h->stream) ||
      cudaStreamSynchronize(h->stream))
    return 100;
  double mx = 0.0;
  for (int b = 0; b < nblocks; ++b) mx = part[b] > mx ? part[b] : mx;
  *out = mx;
  return 0;
}

}  // namespace nmg
