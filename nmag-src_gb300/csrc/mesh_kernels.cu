// mesh_kernels.cu -- device-side mesh topology, CSR build and P1 assembly.
//
// Replaces the reference's one-time setup on the host: DOF numbering and
// simplex membership (src/fem.ml:2434-2930), the operator vivificator with
// PETSc MatSetValues(ADD) assembly (fem.ml:4890-5366, nsim.ml:1758), box
// volumes (fem.ml:1757-1790), outer-face detection (fem.ml:2785-2818) and the
// surface triangles / solid angles of the BEM (bem3d.ml:32-181,
// mesh.ml:1792-1821).
//
// This translation unit is compiled with --fmad=false: every floating-point
// expression below is evaluated in the written order without contraction, so
// the CSR values (K, G, D, volumes) are bit-identical to a CPU evaluation in
// the same order.  Each kernel writes one row (or one tet / face) per thread;
// accumulation order is fixed (tets ascending), so results are deterministic.
#include "nmg_internal.h"

namespace nmg {
namespace {

__device__ __forceinline__ void atomic_or_err(int *err, int bit) { atomicOr(err, bit); }

// Barycentric gradients of a tet: rows of the inverse point matrix
// (Simplex.get_inv_point_matrices), and |det| = 6 * volume.
__global__ void k_tet_geom(int T, const double *__restrict__ X, const int32_t *__restrict__ tets,
                           double *__restrict__ dL, double *__restrict__ adet) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int32_t *v = tets + 4 * (size_t)t;
  const double *p0 = X + 3 * (size_t)v[0], *p1 = X + 3 * (size_t)v[1], *p2 = X + 3 * (size_t)v[2],
               *p3 = X + 3 * (size_t)v[3];
  double e1[3], e2[3], e3[3], c23[3], c31[3], c12[3];
  for (int d = 0; d < 3; ++d) { e1[d] = p1[d] - p0[d]; e2[d] = p2[d] - p0[d]; e3[d] = p3[d] - p0[d]; }
  c23[0] = e2[1] * e3[2] - e2[2] * e3[1]; c23[1] = e2[2] * e3[0] - e2[0] * e3[2]; c23[2] = e2[0] * e3[1] - e2[1] * e3[0];
  c31[0] = e3[1] * e1[2] - e3[2] * e1[1]; c31[1] = e3[2] * e1[0] - e3[0] * e1[2]; c31[2] = e3[0] * e1[1] - e3[1] * e1[0];
  c12[0] = e1[1] * e2[2] - e1[2] * e2[1]; c12[1] = e1[2] * e2[0] - e1[0] * e2[2]; c12[2] = e1[0] * e2[1] - e1[1] * e2[0];
  double det = e1[0] * c23[0] + e1[1] * c23[1] + e1[2] * c23[2];
  double inv = 1.0 / det;
  double *o = dL + 12 * (size_t)t;
  for (int d = 0; d < 3; ++d) {
    double a1 = c23[d] * inv, a2 = c31[d] * inv, a3 = c12[d] * inv;
    o[3 + d] = a1; o[6 + d] = a2; o[9 + d] = a3;
    o[d] = -((a1 + a2) + a3);
  }
  adet[t] = fabs(det);
}

__global__ void k_count_vertices(int n4, const int32_t *__restrict__ tets, int32_t *cnt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n4) atomicAdd(&cnt[tets[k]], 1);
}

// Single-block exclusive scan over n ints (out has n+1 entries; out[n] = total).
__global__ void k_exclusive_scan(int n, const int32_t *__restrict__ in, int32_t *__restrict__ out) {
  __shared__ int warp_sums[32];
  __shared__ int carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int base = 0; base < n; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int nw = blockDim.x >> 5;
      int s = lane < nw ? warp_sums[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += y; }
      if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    int prefix = carry_s + (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
    if (i < n) out[i] = prefix;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = prefix + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry_s;
}

__global__ void k_fill_adjacency(int T, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                                 int32_t *fill, int32_t *__restrict__ idx) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  for (int a = 0; a < 4; ++a) {
    int v = tets[4 * (size_t)t + a];
    int slot = atomicAdd(&fill[v], 1);
    idx[ptr[v] + slot] = t;
  }
}

// Sort each node's tet list ascending (the reference keeps a site's simplices
// in ascending order, fem.ml:2523-2577); also flags oversized lists.
__global__ void k_sort_adjacency(int N, const int32_t *__restrict__ ptr, int32_t *__restrict__ idx, int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = ptr[i], hi = ptr[i + 1];
  if (hi - lo > kMaxNodeTets) atomic_or_err(err, ERR_DEGREE);
  for (int a = lo + 1; a < hi; ++a) {
    int key = idx[a], b = a - 1;
    while (b >= lo && idx[b] > key) { idx[b + 1] = idx[b]; --b; }
    idx[b + 1] = key;
  }
}

// Face neighbours: nbr[4t+f] = tet sharing the face opposite local vertex f, or -1.
__global__ void k_face_neighbours(int T, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                                  const int32_t *__restrict__ idx, int32_t *__restrict__ nbr) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 4 * T) return;
  int t = k >> 2, f = k & 3;
  const int32_t *v = tets + 4 * (size_t)t;
  int fv[3], c = 0;
  for (int a = 0; a < 4; ++a) if (a != f) fv[c++] = v[a];
  int vmin = min(fv[0], min(fv[1], fv[2]));
  int found = -1;
  for (int q = ptr[vmin]; q < ptr[vmin + 1]; ++q) {
    int u = idx[q];
    if (u == t) continue;
    const int32_t *w = tets + 4 * (size_t)u;
    int hit = 0;
    for (int b = 0; b < 4; ++b) hit += (w[b] == fv[0]) + (w[b] == fv[1]) + (w[b] == fv[2]);
    if (hit == 3) { found = u; break; }
  }
  nbr[k] = found;
}

__global__ void k_mark_boundary(int T, const int32_t *__restrict__ tets, const int32_t *__restrict__ nbr,
                                int32_t *flag, int32_t *nouter) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 4 * T) return;
  if (nbr[k] >= 0) return;
  atomicAdd(nouter, 1);
  int t = k >> 2, f = k & 3;
  for (int a = 0; a < 4; ++a) if (a != f) flag[tets[4 * (size_t)t + a]] = 1;
}

__global__ void k_boundary_index(int N, const int32_t *__restrict__ flag, const int32_t *__restrict__ scan,
                                 int32_t *__restrict__ b_of_node, int32_t *__restrict__ node_of_b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (flag[i]) { b_of_node[i] = scan[i]; node_of_b[scan[i]] = i; }
  else b_of_node[i] = -1;
}

// Distinct neighbours (incl. self) of node i, ascending, into a fixed buffer.
__device__ int node_neighbours(int i, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                               const int32_t *__restrict__ idx, int32_t *buf, int *err) {
  int n = 0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const int32_t *v = tets + 4 * (size_t)idx[q];
    for (int a = 0; a < 4; ++a) {
      int c = v[a];
      int pos = n;
      while (pos > 0 && buf[pos - 1] > c) --pos;
      if (pos > 0 && buf[pos - 1] == c) continue;
      if (n >= kMaxRowLen) { atomic_or_err(err, ERR_DEGREE); return n; }
      for (int s = n; s > pos; --s) buf[s] = buf[s - 1];
      buf[pos] = c;
      ++n;
    }
  }
  return n;
}

__global__ void k_row_count(int N, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                            const int32_t *__restrict__ idx, int32_t *__restrict__ cnt, int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int32_t buf[kMaxRowLen];
  cnt[i] = node_neighbours(i, tets, ptr, idx, buf, err);
}

__global__ void k_row_fill(int N, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                           const int32_t *__restrict__ idx, const int32_t *__restrict__ row_ptr,
                           int32_t *__restrict__ col_idx, int32_t *__restrict__ diag_pos, int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int32_t buf[kMaxRowLen];
  int n = node_neighbours(i, tets, ptr, idx, buf, err);
  int base = row_ptr[i];
  for (int k = 0; k < n; ++k) {
    col_idx[base + k] = buf[k];
    if (buf[k] == i) diag_pos[i] = base + k;
  }
}

__device__ __forceinline__ int row_find(const int32_t *__restrict__ cols, int lo, int hi, int c) {
  while (lo < hi) { int mid = (lo + hi) >> 1; if (cols[mid] < c) lo = mid + 1; else hi = mid; }
  return lo;
}

// P1 values, one row per thread, tets ascending (see file header):
//   K   += (|det|/6) dL_a . dL_b            <d/dxj a || d/dxj b>
//   G_d += (|det|/24) dL_b[d]               <a || d/dxj b>
//   S_d += (1+delta_ab)(|det|/24) dL_f[d]   outer face f (a,b != f): the D/Dxj term
//   D_d  = G_d + S_d ;  V_i += |det|/24
__global__ void k_values(int N, int nnz, const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                         const int32_t *__restrict__ idx, const double *__restrict__ dL,
                         const double *__restrict__ adet, const int32_t *__restrict__ nbr,
                         const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                         double *__restrict__ K, double *__restrict__ G, double *__restrict__ D,
                         double *__restrict__ vol) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = row_ptr[i], hi = row_ptr[i + 1];
  for (int k = lo; k < hi; ++k) {
    K[k] = 0.0;
    for (int d = 0; d < 3; ++d) { G[(size_t)d * nnz + k] = 0.0; D[(size_t)d * nnz + k] = 0.0; }
  }
  double V = 0.0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    int t = idx[q];
    const int32_t *v = tets + 4 * (size_t)t;
    const double *g = dL + 12 * (size_t)t;
    double ad = adet[t];
    int a = 0;
    while (v[a] != i) ++a;
    double kc = ad / 6.0, gc = ad / 24.0;
    for (int b = 0; b < 4; ++b) {
      int pos = row_find(col_idx, lo, hi, v[b]);
      if (pos >= hi || col_idx[pos] != v[b]) continue;  // only after a reported degree overflow
      K[pos] += kc * ((g[3 * a] * g[3 * b] + g[3 * a + 1] * g[3 * b + 1]) + g[3 * a + 2] * g[3 * b + 2]);
      for (int d = 0; d < 3; ++d) G[(size_t)d * nnz + pos] += gc * g[3 * b + d];
    }
    V += gc;
  }
  vol[i] = V;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    int t = idx[q];
    const int32_t *v = tets + 4 * (size_t)t;
    const double *g = dL + 12 * (size_t)t;
    int a = 0;
    while (v[a] != i) ++a;
    for (int f = 0; f < 4; ++f) {
      if (f == a || nbr[4 * (size_t)t + f] >= 0) continue;
      double sf[3];
      for (int d = 0; d < 3; ++d) sf[d] = (adet[t] / 24.0) * g[3 * f + d];
      for (int b = 0; b < 4; ++b) {
        if (b == f) continue;
        int pos = row_find(col_idx, lo, hi, v[b]);
        if (pos >= hi || col_idx[pos] != v[b]) continue;
        for (int d = 0; d < 3; ++d) D[(size_t)d * nnz + pos] += (a == b) ? (sf[d] + sf[d]) : sf[d];
      }
    }
  }
  for (int k = lo; k < hi; ++k)
    for (int d = 0; d < 3; ++d) D[(size_t)d * nnz + k] = G[(size_t)d * nnz + k] + D[(size_t)d * nnz + k];
}

// Surface triangles by the reference rule (bem3d.ml:83-176): boundary node sb
// (short order), its tets ascending, each opposing vertex; emit the face when
// every other vertex is a boundary node with short index >= sb.
template <bool EMIT>
__global__ void k_triangles(int nb, const int32_t *__restrict__ node_of_b, const int32_t *__restrict__ b_of_node,
                            const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                            const int32_t *__restrict__ idx, const double *__restrict__ dL,
                            int32_t *__restrict__ cnt_or_off, int ntri, int32_t *__restrict__ tri,
                            double *__restrict__ tri_normal) {
  int sb = blockIdx.x * blockDim.x + threadIdx.x;
  if (sb >= nb) return;
  int node = node_of_b[sb];
  int c = 0;
  int base = EMIT ? cnt_or_off[sb] : 0;
  for (int q = ptr[node]; q < ptr[node + 1]; ++q) {
    int t = idx[q];
    const int32_t *v = tets + 4 * (size_t)t;
    int bidx[4], a = -1;
    for (int k = 0; k < 4; ++k) { bidx[k] = b_of_node[v[k]]; if (bidx[k] == sb) a = k; }
    for (int op = 0; op < 4; ++op) {
      if (op == a) continue;
      bool ok = true;
      for (int k = 0; k < 4 && ok; ++k) {
        if (k == op) continue;
        if (bidx[k] < bidx[a]) ok = false; else if (bidx[k] == -1) ok = false;
      }
      if (!ok) continue;
      if (EMIT) {
        int pos = ntri - 1 - (base + c);  // the reference prepends: final order is reversed
        int k3 = 0;
        for (int k = 0; k < 4; ++k) if (k != op) tri[3 * (size_t)pos + k3++] = bidx[k];
        const double *g = dL + 12 * (size_t)t + 3 * op;
        double r = -1.0 / sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        for (int d = 0; d < 3; ++d) tri_normal[3 * (size_t)pos + d] = r * g[d];
      }
      ++c;
    }
  }
  if (!EMIT) cnt_or_off[sb] = c;
}

// snippets.ml:1229-1258 (van Oosterom-Strackee solid angle).
__device__ double space_angle(const double *obs, const double *p0, const double *p1, const double *p2) {
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
  q = q < -1.0 ? -1.0 : (q > 1.0 ? 1.0 : q);
  return 2.0 * acos(q);
}

// Interior solid angle at each boundary node (mesh.ml:1792-1821).
__global__ void k_solid_angles(int nb, const int32_t *__restrict__ node_of_b, const double *__restrict__ X,
                               const int32_t *__restrict__ tets, const int32_t *__restrict__ ptr,
                               const int32_t *__restrict__ idx, double *__restrict__ out) {
  int sb = blockIdx.x * blockDim.x + threadIdx.x;
  if (sb >= nb) return;
  int node = node_of_b[sb];
  double acc = 0.0;
  for (int q = ptr[node]; q < ptr[node + 1]; ++q) {
    const int32_t *v = tets + 4 * (size_t)idx[q];
    int ix0 = 0;
    while (v[ix0] != node) ++ix0;
    int ix1 = ix0 <= 0 ? 1 : 0, ix2 = ix0 <= 1 ? 2 : 1, ix3 = ix0 <= 2 ? 3 : 2;
    acc += fabs(space_angle(X + 3 * (size_t)v[ix0], X + 3 * (size_t)v[ix1], X + 3 * (size_t)v[ix2],
                            X + 3 * (size_t)v[ix3]));
  }
  out[sb] = acc;
}

// ---- reference-shaped operator export (nmag_lam.py:569-606) ----
__global__ void k_export_count(int which, int N, const int32_t *__restrict__ row_ptr,
                               const int32_t *__restrict__ col_idx, const int32_t *__restrict__ b_of_node,
                               int32_t *__restrict__ cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int len = row_ptr[i + 1] - row_ptr[i];
  switch (which) {
    case 0: case 3: cnt[3 * i] = cnt[3 * i + 1] = cnt[3 * i + 2] = len; break;
    case 1: cnt[i] = 3 * len; break;
    case 2: cnt[i] = len; break;
    case 4: case 5: {
      if (b_of_node[i] >= 0) { cnt[i] = (which == 4) ? 1 : 0; break; }
      int c = 0;
      for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        bool bnd = b_of_node[col_idx[k]] >= 0;
        c += (which == 4) ? !bnd : bnd;
      }
      cnt[i] = c;
    } break;
  }
}

__global__ void k_export_fill(int which, int N, int nnz, double coeff, const int32_t *__restrict__ row_ptr,
                              const int32_t *__restrict__ col_idx, const int32_t *__restrict__ b_of_node,
                              const double *__restrict__ K, const double *__restrict__ G,
                              const double *__restrict__ D, const int32_t *__restrict__ out_rp,
                              int32_t *__restrict__ ci, double *__restrict__ va) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = row_ptr[i], hi = row_ptr[i + 1];
  switch (which) {
    case 0:
      for (int c = 0; c < 3; ++c) {
        int o = out_rp[3 * i + c];
        for (int k = lo; k < hi; ++k, ++o) { ci[o] = 3 * col_idx[k] + c; va[o] = coeff * K[k]; }
      }
      break;
    case 1: {
      int o = out_rp[i];
      for (int k = lo; k < hi; ++k)
        for (int d = 0; d < 3; ++d, ++o) { ci[o] = 3 * col_idx[k] + d; va[o] = coeff * D[(size_t)d * nnz + k]; }
    } break;
    case 2: {
      int o = out_rp[i];
      for (int k = lo; k < hi; ++k, ++o) { ci[o] = col_idx[k]; va[o] = coeff * K[k]; }
    } break;
    case 3:
      for (int d = 0; d < 3; ++d) {
        int o = out_rp[3 * i + d];
        for (int k = lo; k < hi; ++k, ++o) { ci[o] = col_idx[k]; va[o] = -coeff * G[(size_t)d * nnz + k]; }
      }
      break;
    case 4: {
      int o = out_rp[i];
      if (b_of_node[i] >= 0) { ci[o] = i; va[o] = 1.0; break; }
      for (int k = lo; k < hi; ++k) {
        if (b_of_node[col_idx[k]] >= 0) continue;
        ci[o] = col_idx[k]; va[o] = -coeff * K[k]; ++o;
      }
    } break;
    case 5: {
      int o = out_rp[i];
      if (b_of_node[i] >= 0) break;
      for (int k = lo; k < hi; ++k) {
        int b = b_of_node[col_idx[k]];
        if (b < 0) continue;
        ci[o] = b; va[o] = coeff * K[k]; ++o;
      }
    } break;
  }
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

namespace {
__global__ void k_recip(int n, const double *__restrict__ a, double *__restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = 1.0 / a[i];
}
}  // namespace

int build_mesh(nmg_handle *h, const double *coords, const int32_t *tets, std::string &err) {
  Mesh &M = h->mesh;
  cudaStream_t s = h->stream;
  const int N = M.N, T = M.T;
  NMG_CUDA_TRY(M.coords.alloc(3 * (size_t)N), "alloc coords");
  NMG_CUDA_TRY(M.tets.alloc(4 * (size_t)T), "alloc tets");
  NMG_CUDA_TRY(cudaMemcpyAsync(M.coords.p, coords, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s), "h2d coords");
  NMG_CUDA_TRY(cudaMemcpyAsync(M.tets.p, tets, sizeof(int32_t) * 4 * T, cudaMemcpyHostToDevice, s), "h2d tets");
  NMG_CUDA_TRY(M.dL.alloc(12 * (size_t)T), "alloc dL");
  NMG_CUDA_TRY(M.adet.alloc(T), "alloc adet");
  k_tet_geom<<<nblk(T, 256), 256, 0, s>>>(T, M.coords, M.tets, M.dL, M.adet);

  DevBuf<int32_t> cnt, fill, flag, scan, scalars;
  NMG_CUDA_TRY(cnt.alloc(N + 1), "alloc");
  NMG_CUDA_TRY(fill.alloc(N), "alloc");
  NMG_CUDA_TRY(scalars.alloc(4), "alloc");
  NMG_CUDA_TRY(M.nt_ptr.alloc(N + 1), "alloc");
  NMG_CUDA_TRY(M.nt_idx.alloc(4 * (size_t)T), "alloc");
  cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (N + 1), s);
  cudaMemsetAsync(fill.p, 0, sizeof(int32_t) * N, s);
  cudaMemsetAsync(scalars.p, 0, sizeof(int32_t) * 4, s);
  cudaMemsetAsync(h->ws.err.p, 0, sizeof(int), s);
  k_count_vertices<<<nblk(4LL * T, 256), 256, 0, s>>>(4 * T, M.tets, cnt);
  k_exclusive_scan<<<1, 1024, 0, s>>>(N, cnt, M.nt_ptr);
  k_fill_adjacency<<<nblk(T, 256), 256, 0, s>>>(T, M.tets, M.nt_ptr, fill, M.nt_idx);
  k_sort_adjacency<<<nblk(N, 256), 256, 0, s>>>(N, M.nt_ptr, M.nt_idx, h->ws.err);
  NMG_CUDA_TRY(M.nbr.alloc(4 * (size_t)T), "alloc nbr");
  k_face_neighbours<<<nblk(4LL * T, 256), 256, 0, s>>>(T, M.tets, M.nt_ptr, M.nt_idx, M.nbr);

  NMG_CUDA_TRY(flag.alloc(N), "alloc");
  NMG_CUDA_TRY(scan.alloc(N + 1), "alloc");
  cudaMemsetAsync(flag.p, 0, sizeof(int32_t) * N, s);
  k_mark_boundary<<<nblk(4LL * T, 256), 256, 0, s>>>(T, M.tets, M.nbr, flag, scalars.p + 1);
  k_exclusive_scan<<<1, 1024, 0, s>>>(N, flag, scan);
  int32_t host_sc[2];
  NMG_CUDA_TRY(cudaMemcpyAsync(&host_sc[0], scan.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "d2h");
  NMG_CUDA_TRY(cudaMemcpyAsync(&host_sc[1], scalars.p + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "d2h");
  NMG_CUDA_TRY(cudaStreamSynchronize(s), "topology");
  M.nb = host_sc[0];
  M.nouter = host_sc[1];
  NMG_CUDA_TRY(M.b_of_node.alloc(N), "alloc");
  NMG_CUDA_TRY(M.node_of_b.alloc(M.nb), "alloc");
  k_boundary_index<<<nblk(N, 256), 256, 0, s>>>(N, flag, scan, M.b_of_node, M.node_of_b);

  // CSR pattern
  k_row_count<<<nblk(N, 128), 128, 0, s>>>(N, M.tets, M.nt_ptr, M.nt_idx, cnt, h->ws.err);
  NMG_CUDA_TRY(M.row_ptr.alloc(N + 1), "alloc");
  k_exclusive_scan<<<1, 1024, 0, s>>>(N, cnt, M.row_ptr);
  int32_t nnz = 0;
  NMG_CUDA_TRY(cudaMemcpyAsync(&nnz, M.row_ptr.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "d2h");
  NMG_CUDA_TRY(cudaStreamSynchronize(s), "csr count");
  M.nnz = nnz;
  NMG_CUDA_TRY(M.col_idx.alloc(nnz), "alloc");
  NMG_CUDA_TRY(M.diag_pos.alloc(N), "alloc");
  k_row_fill<<<nblk(N, 128), 128, 0, s>>>(N, M.tets, M.nt_ptr, M.nt_idx, M.row_ptr, M.col_idx, M.diag_pos, h->ws.err);
  NMG_CUDA_TRY(M.K.alloc(nnz), "alloc K");
  NMG_CUDA_TRY(M.G.alloc(3 * (size_t)nnz), "alloc G");
  NMG_CUDA_TRY(M.D.alloc(3 * (size_t)nnz), "alloc D");
  NMG_CUDA_TRY(M.vol.alloc(N), "alloc vol");
  k_values<<<nblk(N, 128), 128, 0, s>>>(N, nnz, M.tets, M.nt_ptr, M.nt_idx, M.dL, M.adet, M.nbr, M.row_ptr,
                                        M.col_idx, M.K, M.G, M.D, M.vol);
  NMG_CUDA_TRY(M.ivol.alloc(N), "alloc");
  k_recip<<<nblk(N, 256), 256, 0, s>>>(N, M.vol, M.ivol);

  // surface triangles
  DevBuf<int32_t> tcnt, toff;
  NMG_CUDA_TRY(tcnt.alloc(M.nb + 1), "alloc");
  NMG_CUDA_TRY(toff.alloc(M.nb + 1), "alloc");
  k_triangles<false><<<nblk(M.nb, 128), 128, 0, s>>>(M.nb, M.node_of_b, M.b_of_node, M.tets, M.nt_ptr, M.nt_idx,
                                                      M.dL, tcnt, 0, nullptr, nullptr);
  k_exclusive_scan<<<1, 1024, 0, s>>>(M.nb, tcnt, toff);
  int32_t ntri = 0;
  NMG_CUDA_TRY(cudaMemcpyAsync(&ntri, toff.p + M.nb, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "d2h");
  NMG_CUDA_TRY(cudaStreamSynchronize(s), "triangles");
  M.ntri = ntri;
  NMG_CUDA_TRY(M.tri.alloc(3 * (size_t)ntri), "alloc");
  NMG_CUDA_TRY(M.tri_normal.alloc(3 * (size_t)ntri), "alloc");
  k_triangles<true><<<nblk(M.nb, 128), 128, 0, s>>>(M.nb, M.node_of_b, M.b_of_node, M.tets, M.nt_ptr, M.nt_idx,
                                                     M.dL, toff, ntri, M.tri, M.tri_normal);
  NMG_CUDA_TRY(M.solid_angle.alloc(M.nb), "alloc");
  k_solid_angles<<<nblk(M.nb, 128), 128, 0, s>>>(M.nb, M.node_of_b, M.coords, M.tets, M.nt_ptr, M.nt_idx,
                                                  M.solid_angle);
  NMG_CUDA_TRY(cudaGetLastError(), "mesh kernels");
  NMG_CUDA_TRY(cudaStreamSynchronize(s), "mesh build");
  int derr = 0;
  NMG_CUDA_TRY(cudaMemcpy(&derr, h->ws.err.p, sizeof(int), cudaMemcpyDeviceToHost), "d2h err");
  if (derr & ERR_DEGREE) {
    err = "mesh has a node with more neighbours or tets than supported (max 64 / 128)";
    return 3;
  }
  return 0;
}

int export_operator(const nmg_handle *h, int which, double coeff, int *rows, int *cols, int *nnz_out,
                    int32_t *rp, int32_t *ci, double *vals) {
  const Mesh &M = h->mesh;
  cudaStream_t s = h->stream;
  int N = M.N;
  int nr = (which == 0 || which == 3) ? 3 * N : N;
  int nc = (which == 0 || which == 1) ? 3 * N : (which == 5 ? M.nb : N);
  DevBuf<int32_t> cnt, drp, dci;
  DevBuf<double> dva;
  if (cnt.alloc(nr + 1) || drp.alloc(nr + 1)) return 100;
  k_export_count<<<nblk(N, 256), 256, 0, s>>>(which, N, M.row_ptr, M.col_idx, M.b_of_node, cnt);
  k_exclusive_scan<<<1, 1024, 0, s>>>(nr, cnt, drp);
  int32_t total = 0;
  cudaMemcpyAsync(&total, drp.p + nr, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return 100;
  *rows = nr; *cols = nc; *nnz_out = total;
  if (!rp && !ci && !vals) return 0;
  if (dci.alloc(total) || dva.alloc(total)) return 100;
  k_export_fill<<<nblk(N, 256), 256, 0, s>>>(which, N, M.nnz, coeff, M.row_ptr, M.col_idx, M.b_of_node, M.K, M.G,
                                            M.D, drp, dci, dva);
  if (rp) cudaMemcpyAsync(rp, drp.p, sizeof(int32_t) * (nr + 1), cudaMemcpyDeviceToHost, s);
  if (ci) cudaMemcpyAsync(ci, dci.p, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, s);
  if (vals) cudaMemcpyAsync(vals, dva.p, sizeof(double) * total, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : 100;
}

}  // namespace nmg
