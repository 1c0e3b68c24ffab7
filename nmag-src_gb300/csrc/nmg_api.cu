// nmg_api.cu -- the extern "C" boundary of libnmaggpu.so (declared in
// include/nmag_gpu.h).  Argument checking, handle lifetime, host<->device
// copies and error reporting; the numerical work is in the *_kernels.cu files.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "nmg_internal.h"

namespace {
thread_local std::string g_create_error;

int fail(nmg_handle *h, int code, const std::string &msg) {
  if (h) h->last_error = msg;
  else g_create_error = msg;
  return code;
}

bool finite_material(const nmg_material *m) {
  const double v[] = {m->Ms, m->exch_coeff, m->C1, m->C2, m->C3, m->K1, m->axis[0], m->axis[1], m->axis[2],
                      m->anis_coeff, m->E_coeff_half, m->E_coeff_ext};
  for (double x : v)
    if (!(x == x) || x > 1e300 || x < -1e300) return false;
  return true;
}
}  // namespace

namespace nmg {
void set_handleless_error(const std::string &msg) { g_create_error = msg; }
}  // namespace nmg

extern "C" {

int nmg_version(void) { return NMG_VERSION; }

int nmg_set_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
    return fail(nullptr, -1, "nmg_set_device: no such CUDA device");
  return cudaSetDevice(device) == cudaSuccess ? 0 : fail(nullptr, 101, "nmg_set_device: cudaSetDevice failed");
}

const char *nmg_last_error(const nmg_handle *h) { return h ? h->last_error.c_str() : g_create_error.c_str(); }

int nmg_create(const double *coords, int n_nodes, const int32_t *tets, int n_tets, const nmg_material *mat,
               const nmg_options *opt, nmg_handle **out) {
  if (!out) return fail(nullptr, -1, "nmg_create: out is NULL");
  *out = nullptr;
  if (!coords || !tets || !mat) return fail(nullptr, -1, "nmg_create: NULL input array");
  if (n_nodes < 4 || n_tets < 1) return fail(nullptr, -2, "nmg_create: need at least 4 nodes and 1 tetrahedron");
  for (long long k = 0; k < 4LL * n_tets; ++k)
    if (tets[k] < 0 || tets[k] >= n_nodes) return fail(nullptr, -3, "nmg_create: tetrahedron refers to a missing node");
  for (long long k = 0; k < 3LL * n_nodes; ++k)
    if (!(coords[k] == coords[k])) return fail(nullptr, -4, "nmg_create: non-finite coordinate");
  if (!finite_material(mat)) return fail(nullptr, -5, "nmg_create: non-finite material constant");
  if (mat->Ms == 0.0) return fail(nullptr, -5, "nmg_create: Ms must be non-zero");
  if (opt && (opt->n_members < 0 || opt->n_members > nmg::kMaxMembers))
    return fail(nullptr, -6, "nmg_create: n_members must be in [0, " + std::to_string(nmg::kMaxMembers) + "]");
  if (opt && !(opt->bem_anchor_tol >= 0.0 && opt->bem_anchor_tol <= 1e300))
    return fail(nullptr, -6, "nmg_create: bem_anchor_tol must be finite and non-negative");
  if (opt && (opt->bem_precision < 0 || opt->bem_precision > 3))
    return fail(nullptr, -6, "nmg_create: bem_precision must be 0, 1, 2 or 3");
  if (opt && opt->bem_anchor_tol > 0.0 && opt->bem_precision != 2)
    return fail(nullptr, -6, "nmg_create: bem_anchor_tol applies to the compensated product (bem_precision 2)");
  if (opt && (opt->jv_precision < 0 || opt->jv_precision > 1))
    return fail(nullptr, -6, "nmg_create: jv_precision must be 0 or 1");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(nullptr, 101, "nmg_create: no CUDA device");
  nmg_handle *h = new nmg_handle();
  h->mat = *mat;
  if (opt) h->opt = *opt;
  else {
    h->opt.do_demag = 1;
    h->opt.nbc_rtol = h->opt.dbc_rtol = 1e-5;
    h->opt.nbc_atol = h->opt.dbc_atol = 1e-50;
    h->opt.nbc_maxits = h->opt.dbc_maxits = 10000;
  }
  h->nrep = h->opt.n_members > 1 ? h->opt.n_members : 1;
  cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return fail(nullptr, 101, "nmg_create: stream creation failed");
  }
  h->mesh.N = n_nodes;
  h->mesh.T = n_tets;
  std::string err;
  if (h->ws.err.alloc(1) != cudaSuccess) err = "alloc";
  else cudaMemsetAsync(h->ws.err.p, 0, sizeof(int), h->stream);
  int rc = err.empty() ? nmg::build_mesh(h, coords, tets, err) : 100;
  if (!rc) rc = nmg::init_workspace(h, err);
  if (!rc && h->opt.do_demag) rc = nmg::fill_bem(h, err);
  if (rc) {
    g_create_error = "nmg_create: " + err;
    nmg_destroy(h);
    return rc;
  }
  *out = h;
  return 0;
}

int nmg_destroy(nmg_handle *h) {
  if (!h) return -1;
  if (h->stream) cudaStreamSynchronize(h->stream);
  nmg::ts_destroy(h->ts);
  h->ts = nullptr;
  nmg::tape_free(h);
  nmg_handle *pot = h->pot;
  if (h->ws.aux) {   // the mixed-precision CG's auxiliary stream and its events
    cudaStreamSynchronize(h->ws.aux);
    for (cudaEvent_t ev : h->ws.ev_ldl) if (ev) cudaEventDestroy(ev);
    if (h->ws.ev_cg) cudaEventDestroy(h->ws.ev_cg);
    cudaStreamDestroy(h->ws.aux);
  }
  if (h->stream && h->own_stream) cudaStreamDestroy(h->stream);
  delete h;  // member destructors release the device buffers
  if (pot) nmg_destroy(pot);   // several materials: the potential mesh's handle (and the shared stream)
  return 0;
}

int nmg_mesh_info(const nmg_handle *h, int64_t info[6]) {
  if (!h || !info) return -1;
  info[0] = h->mesh.N; info[1] = h->mesh.T; info[2] = h->mesh.nnz;
  info[3] = h->mesh.nb; info[4] = h->mesh.ntri; info[5] = h->mesh.nouter;
  return 0;
}

static int d2h(const nmg_handle *h, void *dst, const void *src, size_t bytes) {
  if (!dst || !bytes) return 0;
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) return 100;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? 0 : 100;
}

int nmg_get_csr(const nmg_handle *h, int32_t *row_ptr, int32_t *col_idx, double *K, double *G3, double *D3,
                double *vol) {
  if (!h) return -1;
  const nmg::Mesh &M = h->mesh;
  int rc = d2h(h, row_ptr, M.row_ptr.p, sizeof(int32_t) * (M.N + 1));
  rc |= d2h(h, col_idx, M.col_idx.p, sizeof(int32_t) * M.nnz);
  rc |= d2h(h, K, M.K.p, sizeof(double) * M.nnz);
  rc |= d2h(h, G3, M.G.p, sizeof(double) * 3 * (size_t)M.nnz);
  rc |= d2h(h, D3, M.D.p, sizeof(double) * 3 * (size_t)M.nnz);
  rc |= d2h(h, vol, M.vol.p, sizeof(double) * M.N);
  return rc;
}

int nmg_export_operator(const nmg_handle *h, int which, double coeff, int *rows, int *cols, int *nnz,
                        int32_t *row_ptr, int32_t *col_idx, double *vals) {
  if (!h || !rows || !cols || !nnz) return -1;
  if (which < 0 || which > 5) return -2;
  return nmg::export_operator(h, which, coeff, rows, cols, nnz, row_ptr, col_idx, vals);
}

int nmg_get_boundary(const nmg_handle *h, int32_t *node_of_b, int32_t *tri, double *tri_normal, double *solid_angle) {
  if (!h) return -1;
  const nmg::Mesh &M = h->mesh;
  int rc = d2h(h, node_of_b, M.node_of_b.p, sizeof(int32_t) * M.nb);
  rc |= d2h(h, tri, M.tri.p, sizeof(int32_t) * 3 * (size_t)M.ntri);
  rc |= d2h(h, tri_normal, M.tri_normal.p, sizeof(double) * 3 * (size_t)M.ntri);
  rc |= d2h(h, solid_angle, M.solid_angle.p, sizeof(double) * M.nb);
  return rc;
}

int nmg_get_bem(const nmg_handle *h, double *out) {
  if (!h || !out) return -1;
  const nmg::Mesh &M = h->mesh;
  if (!M.bem.p) return fail(const_cast<nmg_handle *>(h), 2, "no BEM matrix (demag disabled)");
  // stored row-major with padded row stride ld: one strided 2D copy
  const size_t nb = M.nb;
  cudaError_t e = cudaMemcpy2DAsync(out, sizeof(double) * nb, M.bem.p, sizeof(double) * M.ld, sizeof(double) * nb, nb,
                                    cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(const_cast<nmg_handle *>(h), 100, std::string("BEM copy: ") + cudaGetErrorString(e));
  return 0;
}

int nmg_set_m(nmg_handle *h, const double *m) {
  if (!h || !m) return -1;
  for (long long k = 0; k < 3LL * h->mesh.N * h->nrep; ++k)
    if (!(m[k] == m[k])) return fail(h, -4, "nmg_set_m: non-finite magnetisation");
  if (cudaMemcpyAsync(h->ws.m.p, m, sizeof(double) * 3 * h->mesh.N * h->nrep, cudaMemcpyHostToDevice, h->stream))
    return fail(h, 100, "nmg_set_m: copy failed");
  if (h->ws.m_mark.p &&
      cudaMemcpyAsync(h->ws.m_mark.p, h->ws.m.p, sizeof(double) * 3 * h->mesh.N * h->nrep, cudaMemcpyDeviceToDevice,
                      h->stream))
    return fail(h, 100, "nmg_set_m: copy failed");
  h->ts_ready = 0;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? 0 : fail(h, 100, "nmg_set_m: sync failed");
}

int nmg_get_m(const nmg_handle *h, double *m) {
  if (!h || !m) return -1;
  return d2h(h, m, h->ws.m.p, sizeof(double) * 3 * h->mesh.N * h->nrep);
}

int nmg_set_h_ext(nmg_handle *h, const double *hx) {
  if (!h || !hx) return -1;
  for (long long k = 0; k < 3LL * h->mesh.N * h->nrep; ++k)
    if (!(hx[k] == hx[k])) return fail(h, -4, "nmg_set_h_ext: non-finite field");
  if (cudaMemcpyAsync(h->ws.h_ext.p, hx, sizeof(double) * 3 * h->mesh.N * h->nrep, cudaMemcpyHostToDevice,
                      h->stream))
    return fail(h, 100, "nmg_set_h_ext: copy failed");
  h->ts_ready = 0;
  return cudaStreamSynchronize(h->stream) == cudaSuccess ? 0 : fail(h, 100, "nmg_set_h_ext: sync failed");
}

int nmg_set_material(nmg_handle *h, const nmg_material *mat) {
  if (!h || !mat) return -1;
  if (!finite_material(mat) || mat->Ms == 0.0) return fail(h, -5, "nmg_set_material: invalid constants");
  h->mat = *mat;
  h->ts_ready = 0;
  return 0;
}

int nmg_set_anisotropy_poly(nmg_handle *h, int n_e, const int32_t *e_pow, const double *e_coef, int n_h,
                            const int32_t *h_pow, const double *h_coef) {
  if (!h) return -1;
  if (h->pot) return fail(h, -2, "nmg_set_anisotropy_poly: not available with several materials");
  if (n_e < 0 || n_h < 0 || n_e > nmg::kAnisMaxTerms || n_h > nmg::kAnisMaxTerms)
    return fail(h, -2, "nmg_set_anisotropy_poly: term counts must be 0.." + std::to_string(nmg::kAnisMaxTerms));
  if ((n_e > 0 && (!e_pow || !e_coef)) || (n_h > 0 && (!h_pow || !h_coef)))
    return fail(h, -1, "nmg_set_anisotropy_poly: null term array");
  auto bad_pow = [](int32_t p) {
    return p < 0 || (p >> 12) != 0 || (p & 15) > nmg::kAnisMaxPow || ((p >> 4) & 15) > nmg::kAnisMaxPow ||
           ((p >> 8) & 15) > nmg::kAnisMaxPow;
  };
  for (int t = 0; t < n_e; ++t)
    if (bad_pow(e_pow[t]) || !std::isfinite(e_coef[t]))
      return fail(h, -2, "nmg_set_anisotropy_poly: bad energy term " + std::to_string(t));
  for (int t = 0; t < n_h; ++t)
    if (bad_pow(h_pow[t]) || !std::isfinite(h_coef[3 * t]) || !std::isfinite(h_coef[3 * t + 1]) ||
        !std::isfinite(h_coef[3 * t + 2]))
      return fail(h, -2, "nmg_set_anisotropy_poly: bad field term " + std::to_string(t));
  nmg::AnisPoly &ap = h->ap;
  ap.ne = ap.nh = 0;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess)   // no launch in flight still reads the old tables
    return fail(h, 100, "nmg_set_anisotropy_poly: sync failed");
  if (ap.epow.alloc(n_e) || ap.ecoef.alloc(n_e) || ap.hpow.alloc(n_h) || ap.hcoef.alloc(3 * (size_t)n_h))
    return fail(h, 100, "nmg_set_anisotropy_poly: device allocation failed");
  // on the handle's (non-blocking) stream, completed before returning
  cudaStream_t s = h->stream;
  if ((n_e > 0 && (cudaMemcpyAsync(ap.epow.p, e_pow, sizeof(int32_t) * n_e, cudaMemcpyHostToDevice, s) ||
                   cudaMemcpyAsync(ap.ecoef.p, e_coef, sizeof(double) * n_e, cudaMemcpyHostToDevice, s))) ||
      (n_h > 0 && (cudaMemcpyAsync(ap.hpow.p, h_pow, sizeof(int32_t) * n_h, cudaMemcpyHostToDevice, s) ||
                   cudaMemcpyAsync(ap.hcoef.p, h_coef, sizeof(double) * 3 * n_h, cudaMemcpyHostToDevice, s))) ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(h, 100, "nmg_set_anisotropy_poly: copy failed");
  ap.ne = n_e;
  ap.nh = n_h;
  h->ts_ready = 0;
  return 0;
}

int nmg_set_stt(nmg_handle *h, double c4, double c5) {
  if (!h) return -1;
  if (h->pot) return fail(h, -2, "nmg_set_stt: not available with several materials");
  if (!std::isfinite(c4) || !std::isfinite(c5)) return fail(h, -5, "nmg_set_stt: non-finite coefficient");
  const size_t n3 = 3 * (size_t)h->mesh.N * h->nrep;
  if ((c4 != 0.0 || c5 != 0.0) && !h->stt.j.p) {   // current density starts at zero
    if (h->stt.j.alloc(n3) || h->stt.dmdc.alloc(n3) ||
        cudaMemsetAsync(h->stt.j.p, 0, sizeof(double) * n3, h->stream) || cudaStreamSynchronize(h->stream))
      return fail(h, 100, "nmg_set_stt: device allocation failed");
  }
  h->stt.c4 = c4;
  h->stt.c5 = c5;
  h->ts_ready = 0;
  return 0;
}

int nmg_set_current_density(nmg_handle *h, const double *j) {
  if (!h) return -1;
  if (h->pot) return fail(h, -2, "nmg_set_current_density: not available with several materials");
  const size_t n3 = 3 * (size_t)h->mesh.N * h->nrep;
  if (j)
    for (size_t k = 0; k < n3; ++k)
      if (!std::isfinite(j[k])) return fail(h, -4, "nmg_set_current_density: non-finite value");
  if (!h->stt.j.p && (h->stt.j.alloc(n3) || h->stt.dmdc.alloc(n3)))
    return fail(h, 100, "nmg_set_current_density: device allocation failed");
  cudaError_t e = j ? cudaMemcpyAsync(h->stt.j.p, j, sizeof(double) * n3, cudaMemcpyHostToDevice, h->stream)
                    : cudaMemsetAsync(h->stt.j.p, 0, sizeof(double) * n3, h->stream);
  if (e != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess)
    return fail(h, 100, "nmg_set_current_density: copy failed");
  h->ts_ready = 0;
  return 0;
}

int nmg_set_pinning(nmg_handle *h, const double *pin) {
  if (!h) return -1;
  const int N = h->mesh.N;
  if (!pin) {   // 1 everywhere: no factor
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(h, 100, "nmg_set_pinning: sync failed");
    h->pin.release();
    h->ts_ready = 0;
    return 0;
  }
  for (int i = 0; i < N; ++i)
    if (!std::isfinite(pin[i])) return fail(h, -4, "nmg_set_pinning: non-finite value");
  if (!h->pin.p && h->pin.alloc(N)) return fail(h, 100, "nmg_set_pinning: device allocation failed");
  if (cudaMemcpyAsync(h->pin.p, pin, sizeof(double) * N, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return fail(h, 100, "nmg_set_pinning: copy failed");
  h->ts_ready = 0;
  return 0;
}

int nmg_eval_fields(nmg_handle *h, double *fields, double *scalars) {
  if (!h) return -1;
  int rc = nmg::rhs_eval(h, h->ws.m, h->ws.dmdt);
  if (rc) return fail(h, rc, "nmg_eval_fields: launch failed");
  rc = nmg::check_device_error(h, "nmg_eval_fields");
  if (rc) return rc;
  const size_t N = (size_t)h->mesh.N * h->nrep, n3 = 3 * N;
  if (fields) {
    const double *src[5] = {h->ws.h_exch, h->ws.h_demag, h->ws.h_anis, h->ws.h_total, h->ws.dmdt};
    for (int k = 0; k < 5; ++k)
      if (d2h(h, fields + k * n3, src[k], sizeof(double) * n3)) return fail(h, 100, "copy failed");
  }
  if (scalars) {
    if (d2h(h, scalars, h->ws.phi.p, sizeof(double) * N) || d2h(h, scalars + N, h->ws.rho.p, sizeof(double) * N))
      return fail(h, 100, "copy failed");
  }
  int it[2] = {0, 0};
  d2h(h, it, h->ws.iters.p, sizeof(it));
  h->last_iters_nbc = it[0];
  h->last_iters_dbc = it[1];
  return 0;
}

int nmg_energy_density(nmg_handle *h, double *E5) {
  if (!h || !E5) return -1;
  if (nmg::energy_density(h, h->ws.m, h->ws.E5)) return fail(h, 100, "energy launch failed");
  return d2h(h, E5, h->ws.E5.p, sizeof(double) * 5 * h->mesh.N * h->nrep);
}

int nmg_averages(nmg_handle *h, double avg_m[3], double energies[5]) {
  if (!h || !avg_m) return -1;
  return nmg::averages(h, h->ws.m, avg_m, energies);
}

int nmg_member_averages(nmg_handle *h, int member, double avg_m[3], double energies[5]) {
  if (!h || !avg_m) return -1;
  if (member < 0 || member >= h->nrep) return fail(h, -2, "nmg_member_averages: member out of range");
  return nmg::averages(h, h->ws.m, avg_m, energies, member);
}

int nmg_ts_init(nmg_handle *h, double t0, double rtol, double atol, int max_order, int krylov_max) {
  if (!h) return -1;
  if (!(rtol > 0.0) || !(atol > 0.0)) return fail(h, -2, "nmg_ts_init: tolerances must be positive");
  if (max_order < 1 || max_order > 5) return fail(h, -2, "nmg_ts_init: max_order must be 1..5");
  if (krylov_max < 1) return fail(h, -2, "nmg_ts_init: krylov_max must be >= 1");
  if (!h->ts || !nmg::ts_matches(h->ts, max_order, krylov_max)) {
    nmg::ts_destroy(h->ts);
    h->ts = nmg::ts_create(h, max_order, krylov_max, rtol, atol);
    if (!h->ts) return fail(h, 100, "nmg_ts_init: out of device memory for the integrator");
  }
  nmg::ts_set_tolerances(h->ts, rtol, atol);
  int rc = nmg::ts_init(h, t0);
  if (rc) return rc;
  return 0;
}

int nmg_ts_advance(nmg_handle *h, double t_final, int exact_tstop, int64_t max_steps, double *t_reached,
                   nmg_ts_stats *stats) {
  if (!h || !t_reached) return -1;
  if (!h->ts || !h->ts_ready) return fail(h, -3, "nmg_ts_advance: timestepper not initialised");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, h->stream);
  int rc = nmg::ts_advance(h, t_final, exact_tstop, max_steps, t_reached, stats);
  cudaEventRecord(e1, h->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  h->timings[0] = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    if (h->last_error.empty()) h->last_error = "nmg_ts_advance failed";
    h->ts_ready = 0;
  }
  return rc;
}

int nmg_max_dm(nmg_handle *h, const double *m_prev, double *out) {
  if (!h || !m_prev || !out) return -1;
  nmg::DevBuf<double> tmp;
  if (tmp.alloc(3 * (size_t)h->mesh.N * h->nrep)) return 100;
  cudaMemcpyAsync(tmp.p, m_prev, sizeof(double) * 3 * h->mesh.N * h->nrep, cudaMemcpyHostToDevice, h->stream);
  return nmg::max_dm(h, h->ws.m, tmp, out);
}

int nmg_max_dm_step(nmg_handle *h, double *out) {
  if (!h || !out) return -1;
  const size_t n3 = 3 * (size_t)h->mesh.N * h->nrep;
  *out = 0.0;
  if (!h->ws.m_mark.p) {
    if (h->ws.m_mark.alloc(n3)) return fail(h, 100, "nmg_max_dm_step: device allocation failed");
  } else {
    int rc = nmg::max_dm(h, h->ws.m, h->ws.m_mark, out);
    if (rc) return fail(h, rc, "nmg_max_dm_step: reduction failed");
  }
  if (cudaMemcpyAsync(h->ws.m_mark.p, h->ws.m.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream))
    return fail(h, 100, "nmg_max_dm_step: copy failed");
  return 0;
}

int nmg_rhs_device(nmg_handle *h, const double *d_m, double *d_dmdt) {
  if (!h || !d_m || !d_dmdt) return -1;
  int rc = nmg::rhs_eval(h, d_m, d_dmdt);
  if (rc) return fail(h, rc, "nmg_rhs_device: launch failed");
  return nmg::check_device_error(h, "nmg_rhs_device");
}

int nmg_bem_apply(nmg_handle *h, const double *d_x, double *d_y, int n_rhs) {
  if (!h || !d_x || !d_y) return -1;
  if (n_rhs < 1) return fail(h, -2, "nmg_bem_apply: n_rhs must be positive");
  if (h->mesh.nb == 0) return fail(h, -2, "nmg_bem_apply: the mesh has no boundary");
  if (h->anchored()) return fail(h, -2, "nmg_bem_apply: not available with the anchored product (bem_anchor_tol)");
  const size_t nb = h->mesh.nb;
  if (h->opt.bem_precision == 3) {
    if (nmg::bem_tc(h, d_x, d_y, n_rhs)) return fail(h, 100, "nmg_bem_apply: " + h->last_error);
  } else {
    for (int n = 0; n < n_rhs; ++n) nmg::bem_gemv(h, d_x + n * nb, d_y + n * nb);
  }
  if (cudaGetLastError() != cudaSuccess) return fail(h, 100, "nmg_bem_apply: launch failed");
  return nmg::check_device_error(h, "nmg_bem_apply");
}

int nmg_set_jacobian(nmg_handle *h, int level, double demag_rtol) {
  if (!h) return -1;
  if (level < 0 || level > 2) return fail(h, -2, "nmg_set_jacobian: level must be 0, 1 or 2");
  if (!(demag_rtol > 0.0 && demag_rtol < 1.0)) return fail(h, -2, "nmg_set_jacobian: demag_rtol must be in (0, 1)");
  if (level != h->jac_level) nmg::ts_invalidate_setup(h->ts);   // the preconditioner follows the level
  h->jac_level = level;
  h->jac_rtol = demag_rtol;
  return 0;
}

int nmg_jacobian_apply(nmg_handle *h, const double *d_m, const double *d_v, double *d_out) {
  if (!h || !d_m || !d_v || !d_out) return -1;
  h->last_error.clear();
  const int rc = nmg::jacobian_apply(h, d_m, d_v, d_out);
  if (rc && h->last_error.empty()) return fail(h, rc, "nmg_jacobian_apply: launch failed");
  return rc;
}

int nmg_rk4_device(nmg_handle *h, double *d_m, double dt, int nsteps) {
  if (!h || !d_m || nsteps < 0) return -1;
  return nmg::rk4_device(h, d_m, dt, nsteps);
}

int nmg_set_element_params(nmg_handle *h, const double *d_wK, const double *d_wD, const double *d_kappa,
                           const double axis[3]) {
  if (!h || !axis) return -1;
  if (h->pot) return fail(h, -2, "nmg_set_element_params: not available with several materials");
  int rc = nmg::set_element_params(h, d_wK, d_wD, d_kappa, axis);
  return rc ? fail(h, rc, "nmg_set_element_params: " + h->last_error) : 0;
}

int nmg_clear_element_params(nmg_handle *h) {
  if (!h) return -1;
  h->ep.active = 0;
  h->ts_ready = 0;
  return 0;
}

int nmg_rk4_forward(nmg_handle *h, const double *d_m0, double dt, int nsteps, int ckpt_every, const double *d_pulses,
                    int n_pulses, int steps_per_pulse, double *d_m_final, double *d_avg_hist) {
  if (!h || !d_m0 || !d_m_final) return -1;
  if (nsteps < 1 || ckpt_every < 1 || !(dt > 0.0)) return fail(h, -2, "nmg_rk4_forward: need nsteps, ckpt_every >= 1, dt > 0");
  if (n_pulses < 0 || (n_pulses > 0 && (!d_pulses || steps_per_pulse < 1)))
    return fail(h, -2, "nmg_rk4_forward: pulses need a device array and steps_per_pulse >= 1");
  int rc = nmg::rk4_forward(h, d_m0, dt, nsteps, ckpt_every, d_pulses, n_pulses, steps_per_pulse, d_m_final, d_avg_hist);
  return rc ? fail(h, rc, "nmg_rk4_forward: " + h->last_error) : 0;
}

int nmg_rk4_adjoint(nmg_handle *h, const double *d_m_final_bar, const double *d_avg_hist_bar, double *d_m0_bar,
                    double *d_wK_bar, double *d_wD_bar, double *d_kappa_bar, double *d_pulses_bar) {
  if (!h) return -1;
  int rc = nmg::rk4_adjoint(h, d_m_final_bar, d_avg_hist_bar, d_m0_bar, d_wK_bar, d_wD_bar, d_kappa_bar,
                            d_pulses_bar);
  return rc ? fail(h, rc, "nmg_rk4_adjoint: " + h->last_error) : 0;
}

int nmg_get_timings(const nmg_handle *h, double out[8]) {
  if (!h || !out) return -1;
  for (int k = 0; k < 8; ++k) out[k] = h->timings[k];
  return 0;
}

int nmg_profile(nmg_handle *h, int enable) {
  if (!h) return -1;
  if (enable) {
    cudaStreamSynchronize(h->stream);
    h->prof.reset();
  }
  h->prof.enabled = enable != 0;
  return 0;
}

int nmg_profile_read(nmg_handle *h, int kernel, int64_t *launches, double *total_ms) {
  if (!h || !launches || !total_ms || kernel < 0 || kernel >= nmg::Profiler::kKernels) return -1;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return 100;
  h->prof.fold();
  *launches = h->prof.done_n[kernel];
  *total_ms = h->prof.done_ms[kernel];
  return 0;
}

int64_t nmg_launch_count(const nmg_handle *h) { return h ? h->launches : -1; }

int nmg_bem_anchor_stats(const nmg_handle *h, int64_t out[2]) {
  if (!h || !out) return -1;
  long long c[2] = {0, 0};
  if (h->ws.anc_count.p && d2h(h, c, h->ws.anc_count.p, sizeof(c))) return 100;
  out[0] = c[0];
  out[1] = c[1];
  return 0;
}

int nmg_cg_iterations(const nmg_handle *h, int64_t total[2]) {
  if (!h || !total) return -1;
  int it[4] = {0, 0, 0, 0};
  if (d2h(h, it, h->ws.iters.p, sizeof(it))) return 100;
  total[0] = it[2];
  total[1] = it[3];
  return 0;
}

}  // extern "C"

namespace nmg {
void Profiler::fold() {
  if (used > 0) cudaEventSynchronize(pool[2 * (used - 1) + 1]);
  for (int k = 0; k < used; ++k) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, pool[2 * k], pool[2 * k + 1]) == cudaSuccess) {
      done_ms[kernel_of[k]] += t;
      ++done_n[kernel_of[k]];
    }
  }
  used = 0;
}
void Profiler::begin(cudaStream_t s, int kernel, int *slot) {
  *slot = -1;
  if (used >= kMaxPairs) fold();   // a long profiled run: resolve the full pool (one wait) and reuse it
  if (pool.empty()) {
    pool.resize(2 * kMaxPairs);
    for (auto &e : pool) cudaEventCreate(&e);
  }
  kernel_of[used] = kernel;
  cudaEventRecord(pool[2 * used], s);
  *slot = used++;
}
void Profiler::end(cudaStream_t s, int slot) { cudaEventRecord(pool[2 * slot + 1], s); }
Profiler::~Profiler() {
  for (auto &e : pool) cudaEventDestroy(e);
}
}  // namespace nmg
