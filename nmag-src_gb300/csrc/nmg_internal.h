// nmg_internal.h -- internal types of libnmaggpu.so (device buffers, launch
// helpers and the kernels' host-side launchers).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/nmag_gpu.h"

namespace nmg {

// Error flag bits written by device code (never trap): the host turns them
// into a status code and a message.
enum DeviceError : int {
  ERR_NONE = 0,
  ERR_DEGREE = 1,       // a node belongs to more tets than the fixed-size row buffer allows
  ERR_BARRIER = 2,      // a grid barrier gave up waiting (bounded spin)
  ERR_NONFINITE = 4,    // a solver produced NaN/Inf
  ERR_CG_MAXITS = 8,    // CG hit its iteration cap
};

constexpr int kMaxRowLen = 64;     // max distinct neighbours (incl. self) per node
constexpr int kMaxMembers = 256;   // ensemble members per handle
constexpr int kChunk = 8;          // members per CG / BEM launch
constexpr int kMaxNodeTets = 128;  // max tets around one node

template <class T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (!count) return cudaSuccess;
    return cudaMalloc(&p, sizeof(T) * count);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DevBuf() { release(); }
  void swap(DevBuf &o) {
    T *q = p; p = o.p; o.p = q;
    size_t m = n; n = o.n; o.n = m;
  }
  operator T *() const { return p; }
};

// Triangle geometry for the Lindholm evaluation (bem3d_stubs.c:466-525).
struct TriGeo {
  double p[3][3], s_l[3], eta[3][3], zeta_v[3], gam01, gam12, gam20, factor, maxgeo;
  int ok, pad;
};

struct Mesh {
  int N = 0, T = 0, nnz = 0, nb = 0, ntri = 0, nouter = 0;
  DevBuf<double> coords, dL, adet, K, G, D, vol, tri_normal, solid_angle;
  DevBuf<double> ivol;   // 1 / vol (the node kernels multiply instead of dividing)
  DevBuf<int32_t> tets, nt_ptr, nt_idx, nbr, row_ptr, col_idx, diag_pos, b_of_node, node_of_b, tri;
  DevBuf<double> bem;      // FP64 BEM, row-major with padded row stride ld (bem[k*ld + c] = B[k][c])
  DevBuf<float> bem32;     // FP32 copy (precision forms 1, 2), same layout
  DevBuf<uint16_t> bem16lo; // form 2: BF16 bits of B - fp32(B), same layout (B ~ hi + lo to ~2^-32)
  // anchored ensemble product: FP16 bits of B * h16_scale in the m16n8k16
  // A-fragment order, tiles of 16 x 16 (h16_kt tiles per row block)
  DevBuf<uint16_t> bem16f;
  int h16_kt = 0;
  float h16_scale = 1.f;
  int ld = 0;              // row stride: nb rounded up to a multiple of 8 (64-byte aligned FP64 rows)
  DevBuf<TriGeo> trigeo;
  DevBuf<double> obs_max;
};

constexpr int kBasisMax = 10;   // warm-start basis size of the CG solves (kBasis)
// A member's factor of its warm-start Gram system (row i of the unit lower
// factor, 1 / D_i, the kept directions, the basis size it was formed for).
struct GramLDL {
  double L[kBasisMax * kBasisMax];
  double rd[kBasisMax];
  unsigned on;
  int n;
};

struct Workspace {
  DevBuf<double> m, h_ext, h_exch, h_demag, h_anis, h_total, dmdt, rho, phi1, phi2, phi, rhs2;
  DevBuf<double> b1, b2, bpart, cg_r, cg_z, cg_p, cg_q, cg_w, cg_tot, dinv_n, dinv_d, red, E5;
  DevBuf<unsigned> bar;     // grid barrier words: per-block arrival epochs + release epoch
  DevBuf<int> err;          // device error flags
  DevBuf<int> iters;        // CG iterations written by the persistent kernel
  DevBuf<double> basis_b, basis_x, basis_gram;  // CG initial-guess basis per solve kind
  // mixed-precision CG: each basis's Gram factor, formed on the auxiliary
  // stream after a solve for the next solve of that basis; one event per slot
  DevBuf<GramLDL> basis_ldl, ens_basis_ldl;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_cg = nullptr;
  std::vector<cudaEvent_t> ev_ldl;
  DevBuf<int> basis_ring;
  // ensemble: a basis per solve kind and member ([kind][member][kBasis][N])
  DevBuf<double> ens_basis_b, ens_basis_x, ens_basis_gram;
  DevBuf<int> ens_basis_ring;
  DevBuf<int32_t> perm, prow, pcol, pbnd;     // CG solver ordering (spatially binned nodes)
  DevBuf<double> pK, xperm, ainv, rc;         // K in that order, iterate, coarse inverse, coarse residual
  DevBuf<float> ainv32, rc32, z32, rw32;      // FP32 copies / vectors of the mixed-precision CG
  DevBuf<int32_t> mcol, mmid;                 // the mixed-precision CG's shared-memory row order
  DevBuf<double> mK;                          //   its values, modes 0 and 1 (2 x nnz)
  DevBuf<float> mK32;                         //   and their FP32 copies
  int cg_smem_mp = 0;                         // dynamic shared memory of the mixed-precision CG
  int nc = 0;                                 // aggregates of the two-level Neumann CG (0: none)
  int cg_blocks = 0;
  int cg_smem_bytes = 0;     // >0: shared-memory CG (one row per thread)
  int cg_nnz_cap = 0;
  // BEM product decomposition: gemv_blocks blocks; each warp streams seg
  // 32-byte units of the flattened row-major matrix and stores at most maxr
  // row partials (index [0] FP64 matrix, [1] FP32 matrix)
  int gemv_blocks = 1;
  long long gemv_seg[2] = {1, 1};
  int gemv_maxr[2] = {1, 1};
  size_t gemv_x32_off = 0;   // offset (doubles) of the padded FP32 x inside bpart
  // anchored compensated product: per member the anchor x0 and y0 = B x0
  // (member-major like b1 / b2); per chunk [flag, valid]; drift maxima;
  // counters [products, refreshes]
  DevBuf<double> anc_x, anc_y;
  DevBuf<unsigned long long> anc_mx;
  DevBuf<int> anc_flag;
  DevBuf<long long> anc_count;
  // m at the last nmg_max_dm_step / nmg_set_m (allocated on first use)
  DevBuf<double> m_mark;
  // FP16 fragment product: x - x0 of 8 members in B-fragment order, the
  // per-member power-of-two scales, the warps' row-block partials
  DevBuf<uint16_t> x16f;
  DevBuf<float> x16scale, h16part;
  int h16_blocks = 0, h16_maxr = 0;
  long long h16_seg = 0;
};

// Tensor-core BEM product (bem_precision 3): three BF16 planes of B (rows
// padded to Mpad, columns to ldk; plane p at p * Mpad rows), the right-hand
// sides' planes (Rcap rows each), the FP32 per-split partials and the TMA
// tensor maps (CUtensorMap, 128 bytes) over the two plane sets.
struct TcState {
  int Mpad = 0, ldk = 0, nt = 0, Rcap = 0;
  int failed = 0;   // a product could not be formed (host-side set-up); rhs_eval reports it
  DevBuf<uint16_t> bplanes, xplanes;
  DevBuf<float> part;
  alignas(64) unsigned char mapA[128];
  alignas(64) unsigned char mapX[128];
};

// Several magnetic materials (nmag_lam.py:183-330): every material X has its
// own m_X on its sites -- the nodes of the simplices of the regions carrying
// X.  The handle's mesh is then the site mesh, the disjoint union of the
// materials' sub-meshes (sites numbered material by material, nodes
// ascending within a material): its exchange operator, box volumes and weak
// divergence (with the surface term where X ends) are X's own, block by
// block.  The potential lives on the nodes of the whole magnetic mesh, held
// by an inner handle (pot) that owns the Poisson solves and the BEM.
struct SiteMat {   // one material's coefficients (nmg_material, simulation units)
  double Ms, c_exch, C1, C2, C3, K1, ax, ay, az, anis, E_half, E_ext;
};
struct Sites {
  int n_mats = 0;
  std::vector<int> offset, count;     // sites of material k: [offset[k], offset[k] + count[k])
  DevBuf<int32_t> site_node, site_mat; // per site: node of the magnetic mesh, material
  DevBuf<int32_t> node_ptr, node_sites; // node -> its sites (CSR, sites ascending)
  DevBuf<SiteMat> mtab;                // per material
  // local magnetic coupling between materials sharing a node (nmag_lam.py:
  // 16-62): lc[2 (X n_mats + Y)] = the field coefficient of m_Y in H_lc_X,
  // lc[... + 1] the energy coefficient of m_X . m_Y in E_lc_X (null: none)
  std::vector<double> lc_host;
  DevBuf<double> lc;
};

struct Integrator;

// CUDA-event brackets around hot-kernel launches (resolved after the run).
struct Profiler {
  static constexpr int kKernels = 6;
  static constexpr int kMaxPairs = 8192;
  bool enabled = false;
  std::vector<cudaEvent_t> pool;   // 2 * kMaxPairs events, created lazily
  int used = 0;
  int kernel_of[kMaxPairs];
  // totals of the pairs already resolved (the pool is folded into these when it fills)
  long long done_n[kKernels] = {0};
  double done_ms[kKernels] = {0.0};
  void begin(cudaStream_t s, int kernel, int *slot);
  void end(cudaStream_t s, int slot);
  void fold();   // wait for the recorded pairs, add them to the totals, empty the pool
  void reset() {
    used = 0;
    for (int k = 0; k < kKernels; ++k) { done_n[k] = 0; done_ms[k] = 0.0; }
  }
  ~Profiler();
};

}  // namespace nmg

namespace nmg {
// Per-element parameters of the differentiation form: the exchange operator
// sum_T wK_T K_T, the divergence operator built from per-element weights wD_T,
// and the per-node anisotropy coefficient from per-element kappa_T.
struct ElemParams {
  int active = 0;
  DevBuf<double> Kx, Dx, anis;   // nnz, 3 x nnz, N
  DevBuf<int32_t> tpos;          // position of entry (j,i) for entry (i,j) of the scalar pattern
  double axis[3] = {0, 0, 1};
};
struct Tape;                     // RK4 checkpoints of the differentiation form (adjoint.cu)
// Anisotropy given as polynomials in m (nsim_anisotropy.ml:207-236): energy
// density terms (ne) and field terms (nh, three coefficients each); exponents
// packed a | b << 4 | c << 8, each at most kAnisMaxPow.
constexpr int kAnisMaxPow = 13;

// Monomial mx^a my^b mz^c of a packed exponent triple from per-node power tables.
__device__ __forceinline__ double anis_monomial(int p, const double *px, const double *py, const double *pz) {
  return px[p & 15] * py[(p >> 4) & 15] * pz[(p >> 8) & 15];
}

__device__ __forceinline__ void anis_powers(double x, double y, double z, double *px, double *py, double *pz) {
  px[0] = py[0] = pz[0] = 1.0;
#pragma unroll
  for (int k = 1; k <= kAnisMaxPow; ++k) {
    px[k] = px[k - 1] * x; py[k] = py[k - 1] * y; pz[k] = pz[k - 1] * z;
  }
}
constexpr int kAnisMaxTerms = 1024;
struct AnisPoly {
  int ne = 0, nh = 0;
  DevBuf<int32_t> epow, hpow;
  DevBuf<double> ecoef, hcoef;   // ne, 3 x nh (term-major)
};
// Spin-transfer torque (Zhang-Li): coefficients LLG_C4 (adiabatic) and LLG_C5
// (non-adiabatic) of the material, the current density (3 per node, all
// members) and the per-RHS dm_dcurrent = (J . grad) m.
struct Stt {
  double c4 = 0.0, c5 = 0.0;
  DevBuf<double> j, dmdc;
  bool on() const { return (c4 != 0.0 || c5 != 0.0) && j.p; }
};
// The demag part of the exact Jacobian (Jacobian level 2): H_demag is linear
// in m, so its derivative along a direction v is the demag field of v itself.
// The pipeline's buffers for v are swapped into the potential handle's
// workspace for those solves, so the RHS's warm starts (previous potentials
// and initial-guess bases) stay as they were; hdv = H_demag(v), 3 per node of
// the potential mesh and member.
struct JacDemag {
  DevBuf<double> rho, phi1, phi2, phi, rhs2, b1, b2;
  DevBuf<double> basis_b, basis_x, basis_gram, ens_basis_b, ens_basis_x, ens_basis_gram;
  DevBuf<int> basis_ring, ens_basis_ring, iters;
  DevBuf<GramLDL> basis_ldl, ens_basis_ldl;
  DevBuf<double> hdv;
  bool ready = false;
};
}  // namespace nmg

struct nmg_handle {
  nmg::Mesh mesh;
  nmg::Workspace ws;
  nmg_material mat{};
  nmg_options opt{};
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::string last_error;
  nmg::Integrator *ts = nullptr;
  int ts_ready = 0;             // integrator initialised for the current m / H_ext / material
  double *h_pinned = nullptr;   // small pinned staging buffer for scalars
  int last_iters_nbc = 0, last_iters_dbc = 0;
  int64_t n_rhs = 0;
  int64_t launches = 0;         // kernels launched by this handle
  double timings[8] = {0};
  nmg::Profiler prof;
  int nrep = 1;                 // ensemble members B (member-major vectors: member b at b * 3N / b * N)
  nmg::ElemParams ep;
  nmg::AnisPoly ap;
  nmg::Stt stt;
  nmg::DevBuf<double> pin;      // per-node factor of dm/dt and of the Jacobian rows (null: 1 everywhere)
  nmg::TcState tc;              // tensor-core BEM product (bem_precision 3)
  nmg::Sites sites;             // several materials: the site layout (n_mats == 0: one material)
  nmg_handle *pot = nullptr;    // several materials: the handle of the potential mesh (owns BEM, CG)
  bool own_stream = true;       // false: the stream belongs to pot
  nmg::Tape *tape = nullptr;
  int anchor_hold = 0;          // >0: anchored BEM product suspended (RK4 tape runs recompute bit for bit)
  int bem_fp32_only = 0;        // >0: the plain FP32 product even where the compensated one is set up
  // Jacobian of the BDF's Newton iteration: 0 the exchange part only (the
  // reference's); 1 also the local terms (anisotropy, the C3 length term,
  // local couplings); 2 also the demag response, from Poisson solves at
  // jac_rtol (one pair per Jacobian-vector product)
  int jac_level = 0;
  double jac_rtol = 1e-3;
  nmg::JacDemag jd;
  // the mixed-precision CG is used by the forward solves or the adjoint's
  bool mixed_cg() const { return opt.cg_precision == 1 || opt.adjoint_cg_precision == 1; }
  bool anchored() const {
    return opt.bem_anchor_tol > 0.0 && opt.bem_precision == 2 && mesh.bem16lo.p && !anchor_hold;
  }
  const double *exch_K() const { return ep.active ? ep.Kx.p : mesh.K.p; }
};

// Bracket one hot-kernel launch with profiler events (no-op when disabled).
#define NMG_PROF_BEGIN(h, kernel) \
  int prof_slot__ = -1;           \
  if ((h)->prof.enabled) (h)->prof.begin((h)->stream, kernel, &prof_slot__)
#define NMG_PROF_END(h) \
  if (prof_slot__ >= 0) (h)->prof.end((h)->stream, prof_slot__)

namespace nmg {
// Compensated FP32 multiply-add of the BEM products: (S, C) += (h + l)(a + b)
// with h*a split exactly by an FMA, the second-order terms h*b + l*a added to
// the error term, and S updated by TwoSum (~44 bits in FP32 operations).
__device__ __forceinline__ void df_madd(float h, float l, float a, float b, float &S, float &C) {
  const float p = __fmul_rn(h, a);
  const float e = fmaf(h, a, -p);
  const float t = fmaf(h, b, fmaf(l, a, e));
  const float s2 = __fadd_rn(S, p);
  const float bb = __fsub_rn(s2, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s2, bb)), __fsub_rn(p, bb));
  S = s2;
  C += err + t;
}
}  // namespace nmg

namespace nmg {
// ---- launchers (mesh_kernels.cu) ----
int build_mesh(nmg_handle *h, const double *coords, const int32_t *tets, std::string &err);
int export_operator(const nmg_handle *h, int which, double coeff, int *rows, int *cols, int *nnz,
                    int32_t *rp, int32_t *ci, double *vals);
// ---- bem_kernels.cu ----
int fill_bem(nmg_handle *h, std::string &err);
void bem_gemv(nmg_handle *h, const double *x, double *y);
// ---- nmg_sites.cu (several materials) ----
int rhs_eval_sites(nmg_handle *h, const double *d_m, double *d_dmdt);
int energy_density_sites(nmg_handle *h, const double *d_m, double *d_E5);
// ---- rhs_kernels.cu: the demag pipeline from W.rho to W.phi (one handle) ----
int demag_from_rho(nmg_handle *h);
// The exact Jacobian's demag response: h->jd.hdv = H_demag(d_v) for the
// member-major direction d_v (3 per node or site and member); the RHS's
// solver state is left as it was.  demag_response_sites: several materials.
int demag_response(nmg_handle *h, const double *d_v);
int demag_response_sites(nmg_handle *h, const double *d_v);
// J.rho (charges on P's nodes, all members) -> J.phi -> J.hdv, Poisson solves
// at rtol; jac_prepare allocates J (zeroed) for P's workspace once
int jac_prepare(nmg_handle *P, JacDemag &J);
int jac_demag_solve(nmg_handle *P, JacDemag &J, double rtol);
// ---- bem_tc.cu ----
int bem_tc_setup(nmg_handle *h, std::string &err);
int bem_tc(nmg_handle *h, const double *x, double *y, int R);   // Y = B X, R member-major right-hand sides
// ---- rhs_kernels.cu ----
int rhs_eval(nmg_handle *h, const double *d_m, double *d_dmdt);  // full RHS on device vectors
// CG on slot 0/2 (Neumann operator) or 1/3 (Dirichlet operator); slots 2/3
// keep their own warm-start bases.
int cg_solve(nmg_handle *h, int slot, const double *b, double *x, double rtol, double atol, int maxits);
void cg_reset_basis(nmg_handle *h, int slot);
// ---- adjoint.cu ----
void tape_free(nmg_handle *h);
int set_element_params(nmg_handle *h, const double *wK, const double *wD, const double *kappa, const double axis[3]);
int rk4_forward(nmg_handle *h, const double *d_m0, double dt, int nsteps, int ckpt, const double *d_pulses,
                int npulses, int spp, double *d_mT, double *d_hist);
int rk4_adjoint(nmg_handle *h, const double *d_mT_bar, const double *d_hist_bar, double *d_m0_bar, double *d_gwK,
                double *d_gwD, double *d_gkap, double *d_gpul);
int energy_density(nmg_handle *h, const double *d_m, double *d_E5);
int averages(nmg_handle *h, const double *d_m, double avg[3], double energies[5], int member = 0);
int max_dm(nmg_handle *h, const double *d_m, const double *d_mprev, double *out);
int init_workspace(nmg_handle *h, std::string &err);
int check_device_error(nmg_handle *h, const char *where);
// ---- ts (nmg_ts.cu) ----
Integrator *ts_create(nmg_handle *h, int qmax, int maxl, double rtol, double atol);
void ts_destroy(Integrator *t);
bool ts_matches(const Integrator *t, int qmax, int maxl);
void ts_set_tolerances(Integrator *t, double rtol, double atol);
void ts_invalidate_setup(Integrator *t);
int ts_init(nmg_handle *h, double t0);
int ts_advance(nmg_handle *h, double tout, int exact_tstop, int64_t max_steps, double *t_reached,
               nmg_ts_stats *st);
int rk4_device(nmg_handle *h, double *d_m, double dt, int nsteps);
int jacobian_apply(nmg_handle *h, const double *d_m, const double *d_v, double *d_out);
// ---- nmg_api.cu ----
void set_handleless_error(const std::string &msg);  // what nmg_last_error(NULL) reports
}  // namespace nmg

#define NMG_CUDA_TRY(expr, msg)                                                    \
  do {                                                                             \
    cudaError_t e__ = (expr);                                                      \
    if (e__ != cudaSuccess) {                                                      \
      err = std::string(msg) + ": " + cudaGetErrorString(e__);                     \
      return 100;                                                                  \
    }                                                                              \
  } while (0)
