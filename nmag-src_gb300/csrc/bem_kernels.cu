// bem_kernels.cu -- dense Lindholm double-layer BEM on the device.
//
// Replaces the reference's BEM fill: nas_partially_fill_bem_matrix_row_constrained
// (src/bem3d.ml:938-1047) driving caml_bem3d_raw_lindholm_block_pbc
// (src/bem3d_stubs.c:413-610) for every (surface triangle, observer row), then
// adding Omega_i/(4 pi) - 1 on the diagonal (bem3d.ml:1040-1043).
//
// Layout: the fill accumulates into a column-major buffer, a[c*nb + k] =
// B[k][c] (k = observer row, c = boundary column).  One thread owns one
// observer row and walks the triangles in the reference's order, so every
// entry is accumulated in exactly the reference's order with no atomics, and a
// warp's 32 rows are adjacent in memory (coalesced read-modify-write).  A tiled
// transpose then stores the matrix row-major with the row stride padded to a
// multiple of 8 (bem[k*ld + c]), the layout the matrix-vector product streams.
// Compiled with --fmad=false to follow the written operation order.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

#include "nmg_internal.h"

namespace nmg {
namespace {

constexpr double kPi = 3.141592653589793;

// Per-triangle constants of the Lindholm formula (bem3d_stubs.c:466-525).
__global__ void k_tri_setup(int ntri, const int32_t *__restrict__ tri, const double *__restrict__ tri_normal,
                            const int32_t *__restrict__ node_of_b, const double *__restrict__ X,
                            TriGeo *__restrict__ geo) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntri) return;
  TriGeo g;
  double s[3][3], xi[3][3];
  g.ok = 0;
  g.maxgeo = 0.0;
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 3; ++d) {
      g.p[k][d] = X[3 * (size_t)node_of_b[tri[3 * (size_t)t + k]] + d];
      double ax = fabs(g.p[k][d]);
      if (ax > g.maxgeo) g.maxgeo = ax;
    }
  for (int d = 0; d < 3; ++d) {
    s[0][d] = g.p[2][d] - g.p[1][d]; s[1][d] = g.p[0][d] - g.p[2][d]; s[2][d] = g.p[1][d] - g.p[0][d];
  }
  bool ok = true;
  for (int k = 0; k < 3; ++k) {
    g.s_l[k] = sqrt(s[k][0] * s[k][0] + s[k][1] * s[k][1] + s[k][2] * s[k][2]);
    if (g.s_l[k] == 0.0) { ok = false; g.s_l[k] = 1.0; }
    double inv = 1.0 / g.s_l[k];
    for (int d = 0; d < 3; ++d) xi[k][d] = s[k][d] * inv;
  }
  double z[3];
  z[0] = s[1][1] * s[2][2] - s[1][2] * s[2][1];
  z[1] = s[1][2] * s[2][0] - s[1][0] * s[2][2];
  z[2] = s[1][0] * s[2][1] - s[1][1] * s[2][0];
  double len = sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  if (len == 0.0) { ok = false; len = 1.0; }
  double area = 0.5 * len, inv = 1.0 / len;
  for (int d = 0; d < 3; ++d) g.zeta_v[d] = z[d] * inv;
  g.gam01 = xi[0][0] * xi[1][0] + xi[0][1] * xi[1][1] + xi[0][2] * xi[1][2];
  g.gam12 = xi[1][0] * xi[2][0] + xi[1][1] * xi[2][1] + xi[1][2] * xi[2][2];
  g.gam20 = xi[2][0] * xi[0][0] + xi[2][1] * xi[0][1] + xi[2][2] * xi[0][2];
  for (int k = 0; k < 3; ++k) {
    const double *zv = g.zeta_v;
    g.eta[k][0] = zv[1] * xi[k][2] - zv[2] * xi[k][1];
    g.eta[k][1] = zv[2] * xi[k][0] - zv[0] * xi[k][2];
    g.eta[k][2] = zv[0] * xi[k][1] - zv[1] * xi[k][0];
  }
  double f = 1.0 * (1.0 / (8.0 * kPi * area));
  const double *n = tri_normal + 3 * (size_t)t;
  if (g.zeta_v[0] * n[0] + g.zeta_v[1] * n[1] + g.zeta_v[2] * n[2] < 0.0) f = -f;
  g.factor = f;
  g.ok = ok ? 1 : 0;
  geo[t] = g;
}

// Running maximum of |observer coordinate| in row order: the reference's
// geo_eps = 1e-13 * max over the triangle and the observers visited so far
// within one block call (bem3d_stubs.c:531-533).
__global__ void k_observer_prefix_max(int nb, const int32_t *__restrict__ node_of_b, const double *__restrict__ X,
                                      double *__restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double run = 0.0;
  for (int k = 0; k < nb; ++k) {
    const double *o = X + 3 * (size_t)node_of_b[k];
    for (int d = 0; d < 3; ++d) { double a = fabs(o[d]); if (a > run) run = a; }
    out[k] = run;
  }
}

__global__ void __launch_bounds__(128) k_bem_fill(int nb, int ntri, const TriGeo *__restrict__ geo,
                                                  const int32_t *__restrict__ tri,
                                                  const int32_t *__restrict__ node_of_b,
                                                  const double *__restrict__ X, const double *__restrict__ obs_max,
                                                  const double *__restrict__ solid_angle, double *__restrict__ bem) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const double ox = X[3 * (size_t)node_of_b[k]], oy = X[3 * (size_t)node_of_b[k] + 1],
               oz = X[3 * (size_t)node_of_b[k] + 2];
  const double omax = obs_max[k];
  for (int t = 0; t < ntri; ++t) {
    const TriGeo &g = geo[t];
    if (!g.ok) continue;
    double r[3][3], rl[3];
    for (int v = 0; v < 3; ++v) {
      r[v][0] = g.p[v][0] - ox; r[v][1] = g.p[v][1] - oy; r[v][2] = g.p[v][2] - oz;
      rl[v] = sqrt(r[v][0] * r[v][0] + r[v][1] * r[v][1] + r[v][2] * r[v][2]);
    }
    if (rl[0] <= 0.0 || rl[1] <= 0.0 || rl[2] <= 0.0) continue;
    double vlog0 = log((rl[1] + rl[2] + g.s_l[0]) / (rl[1] + rl[2] - g.s_l[0]));
    double vlog1 = log((rl[2] + rl[0] + g.s_l[1]) / (rl[2] + rl[0] - g.s_l[1]));
    double vlog2 = log((rl[0] + rl[1] + g.s_l[2]) / (rl[0] + rl[1] - g.s_l[2]));
    double sp01 = r[0][0] * r[1][0] + r[0][1] * r[1][1] + r[0][2] * r[1][2];
    double sp12 = r[1][0] * r[2][0] + r[1][1] * r[2][1] + r[1][2] * r[2][2];
    double sp20 = r[2][0] * r[0][0] + r[2][1] * r[0][1] + r[2][2] * r[0][2];
    double num = rl[0] * rl[1] * rl[2] + rl[0] * sp12 + rl[1] * sp20 + rl[2] * sp01;
    double den = sqrt(2.0 * (rl[1] * rl[2] + sp12) * (rl[2] * rl[0] + sp20) * (rl[0] * rl[1] + sp01));
    if (den == 0.0) continue;
    double angle = num / den;
    angle = angle < -1.0 ? -1.0 : (angle > 1.0 ? 1.0 : angle);
    angle = 2.0 * acos(angle);
    double zeta = g.zeta_v[0] * r[0][0] + g.zeta_v[1] * r[0][1] + g.zeta_v[2] * r[0][2];
    if (zeta < 0.0) angle = -angle;
    double f = g.factor;
    double geo_eps = (g.maxgeo > omax ? g.maxgeo : omax) * 1e-13;
    if (fabs(zeta) < geo_eps) f = 0.0;
    double gl0 = 1.0 * vlog0 + g.gam01 * vlog1 + g.gam20 * vlog2;
    double gl1 = g.gam01 * vlog0 + 1.0 * vlog1 + g.gam12 * vlog2;
    double gl2 = g.gam20 * vlog0 + g.gam12 * vlog1 + 1.0 * vlog2;
    double e0 = g.eta[0][0] * r[1][0] + g.eta[0][1] * r[1][1] + g.eta[0][2] * r[1][2];
    double e1 = g.eta[1][0] * r[2][0] + g.eta[1][1] * r[2][1] + g.eta[1][2] * r[2][2];
    double e2 = g.eta[2][0] * r[0][0] + g.eta[2][1] * r[0][1] + g.eta[2][2] * r[0][2];
    double lh0 = f * g.s_l[0] * (angle * e0 - zeta * gl0);
    double lh1 = f * g.s_l[1] * (angle * e1 - zeta * gl1);
    double lh2 = f * g.s_l[2] * (angle * e2 - zeta * gl2);
    const int32_t *tv = tri + 3 * (size_t)t;
    bem[(size_t)tv[0] * nb + k] += lh0;
    bem[(size_t)tv[1] * nb + k] += lh1;
    bem[(size_t)tv[2] * nb + k] += lh2;
  }
  bem[(size_t)k * nb + k] += solid_angle[k] / (4.0 * kPi) - 1.0;
}

// Column-major fill buffer (a[c*nb + k]) -> row-major matrix with padded row
// stride ld (b[k*ld + c], pad columns zero), 32x32 tiles through shared memory.
__global__ void k_transpose_pad(int nb, int ld, const double *__restrict__ a, double *__restrict__ b) {
  __shared__ double tile[32][33];
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = c0 + j, k = k0 + threadIdx.x;
    tile[j][threadIdx.x] = (c < nb && k < nb) ? a[(size_t)c * nb + k] : 0.0;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int k = k0 + j, c = c0 + threadIdx.x;
    if (k < nb && c < ld) b[(size_t)k * ld + c] = tile[threadIdx.x][j];
  }
}

// BF16 bits of the FP32 rounding residual B - fp32(B) (round to nearest even).
__global__ void k_split_lo(size_t n, const double *__restrict__ a, const float *__restrict__ hi,
                           uint16_t *__restrict__ lo) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) {
    const __nv_bfloat16 v = __float2bfloat16_rn((float)(a[i] - (double)hi[i]));
    lo[i] = *reinterpret_cast<const uint16_t *>(&v);
  }
}

// FP32 copy of the row-major matrix (same padded stride).
__global__ void k_to_f32(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) b[i] = (float)a[i];
}

// max |B| as float bits (non-negative floats order like their bit patterns).
__global__ void k_absmax_f32(long long n, const float *__restrict__ v, unsigned *__restrict__ out) {
  unsigned m = 0u;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    m = max(m, __float_as_uint(fabsf(v[k])));
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// FP16 copy of B (times scale) in the A-operand fragment order of
// mma.m16n8k16 (row-major): tile (rb, kb) holds rows 16 rb .. +15 and
// columns 16 kb .. +15 as 32 lanes x 8 halves; lane 4 g + t carries
// (g, 2t), (g, 2t+1), (g+8, 2t), (g+8, 2t+1), (g, 2t+8), (g, 2t+9),
// (g+8, 2t+8), (g+8, 2t+9) -- the PTX fragment elements a0..a7 -- so one
// 16-byte load per lane fills the operand.  Entries beyond nb are 0.
__global__ void k_pack_bem16f(int nb, int ld, int KT, long long ntiles, const float *__restrict__ B32, float scale,
                              uint4 *__restrict__ out) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= ntiles * 32) return;
  const long long tile = g >> 5;
  const int lane = (int)(g & 31);
  const int rb = (int)(tile / KT), kb = (int)(tile - (long long)rb * KT);
  const int gq = lane >> 2, t = lane & 3;
  unsigned w[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float v[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = 2 * j + h;
      const int r = 16 * rb + gq + ((i & 2) ? 8 : 0);
      const int c = 16 * kb + 2 * t + (i & 1) + (i >= 4 ? 8 : 0);
      v[h] = (r < nb && c < nb) ? B32[(size_t)r * ld + c] * scale : 0.f;
    }
    const __half2 p = __floats2half2_rn(v[0], v[1]);   // v[0] in the low half
    memcpy(&w[j], &p, sizeof(unsigned));
  }
  out[g] = make_uint4(w[0], w[1], w[2], w[3]);
}

}  // namespace

int fill_bem(nmg_handle *h, std::string &err) {
  Mesh &M = h->mesh;
  cudaStream_t s = h->stream;
  if (M.nb == 0) return 0;
  const size_t nb = M.nb;
  if (M.ld != (M.nb + 7) / 8 * 8) {
    err = "BEM row stride not set up by the workspace";
    return 3;
  }
  NMG_CUDA_TRY(M.trigeo.alloc(M.ntri), "alloc trigeo");
  NMG_CUDA_TRY(M.obs_max.alloc(M.nb), "alloc obs_max");
  {
    // The fill accumulates column-major (coalesced, reference order) into a
    // temporary; one tiled transpose then gives the row-major product layout.
    DevBuf<double> colmajor;
    NMG_CUDA_TRY(colmajor.alloc(nb * nb), "alloc BEM fill buffer (nb^2 doubles)");
    NMG_CUDA_TRY(cudaMemsetAsync(colmajor.p, 0, sizeof(double) * nb * nb, s), "zero BEM");
    k_tri_setup<<<(M.ntri + 127) / 128, 128, 0, s>>>(M.ntri, M.tri, M.tri_normal, M.node_of_b, M.coords, M.trigeo);
    k_observer_prefix_max<<<1, 32, 0, s>>>(M.nb, M.node_of_b, M.coords, M.obs_max);
    k_bem_fill<<<(M.nb + 127) / 128, 128, 0, s>>>(M.nb, M.ntri, M.trigeo, M.tri, M.node_of_b, M.coords, M.obs_max,
                                                   M.solid_angle, colmajor);
    NMG_CUDA_TRY(cudaGetLastError(), "bem fill launch");
    NMG_CUDA_TRY(M.bem.alloc(nb * M.ld), "alloc BEM (nb x ld doubles)");
    dim3 tb(32, 8), tg((M.ld + 31) / 32, (M.nb + 31) / 32);
    k_transpose_pad<<<tg, tb, 0, s>>>(M.nb, M.ld, colmajor, M.bem);
    NMG_CUDA_TRY(cudaGetLastError(), "bem transpose launch");
    NMG_CUDA_TRY(cudaStreamSynchronize(s), "bem fill");
  }
  if (h->opt.bem_precision == 3) {   // tensor-core product: BF16 planes of the FP64 matrix
    if (int rc = bem_tc_setup(h, err)) return rc;
  }
  if (h->opt.bem_precision == 1 || h->opt.bem_precision == 2) {
    NMG_CUDA_TRY(M.bem32.alloc(nb * M.ld), "alloc FP32 BEM");
    k_to_f32<<<h->sm_count * 8, 256, 0, s>>>(nb * M.ld, M.bem, M.bem32);
  }
  if (h->opt.bem_precision == 2) {
    NMG_CUDA_TRY(M.bem16lo.alloc(nb * M.ld), "alloc BEM residual (BF16)");
    k_split_lo<<<h->sm_count * 8, 256, 0, s>>>(nb * M.ld, M.bem, M.bem32, M.bem16lo);
  }
  if (h->opt.bem_precision == 2 && h->opt.bem_anchor_tol > 0.0 && h->nrep > 1 && h->opt.anchor_product == 1) {
    // FP16 fragment copy for the anchored ensemble product, scaled by a power
    // of two that puts max|B| in [2^13, 2^14) (FP16 normal range for the rest)
    DevBuf<unsigned> amax;
    NMG_CUDA_TRY(amax.alloc(1), "alloc");
    NMG_CUDA_TRY(cudaMemsetAsync(amax.p, 0, sizeof(unsigned), s), "zero");
    k_absmax_f32<<<h->sm_count * 4, 256, 0, s>>>((long long)nb * M.ld, M.bem32, amax);
    unsigned bits = 0;
    NMG_CUDA_TRY(cudaMemcpyAsync(&bits, amax.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "copy");
    NMG_CUDA_TRY(cudaStreamSynchronize(s), "absmax");
    float mx;
    std::memcpy(&mx, &bits, sizeof(float));
    int e = 0;
    if (mx > 0.f && std::isfinite(mx)) std::frexp(mx, &e);
    M.h16_scale = std::ldexp(1.f, 14 - e);
    M.h16_kt = (nb + 15) / 16;
    const long long ntiles = (long long)M.h16_kt * M.h16_kt;   // row blocks = column tiles
    NMG_CUDA_TRY(M.bem16f.alloc((size_t)ntiles * 256), "alloc FP16 fragment BEM");
    k_pack_bem16f<<<(unsigned)((ntiles * 32 + 255) / 256), 256, 0, s>>>(
        nb, M.ld, M.h16_kt, ntiles, M.bem32, M.h16_scale, reinterpret_cast<uint4 *>(M.bem16f.p));
    NMG_CUDA_TRY(cudaGetLastError(), "pack FP16 fragment BEM");
  }
  NMG_CUDA_TRY(cudaStreamSynchronize(s), "bem fill");
  return 0;
}

}  // namespace nmg
