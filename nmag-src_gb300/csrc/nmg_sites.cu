// nmg_sites.cu -- several magnetic materials (interface/nmag/nmag_lam.py:
// 183-470, 587-606, 734-832; region -> material mapping main.py:1182-1191).
//
// Every material X has its own magnetisation m_X on its sites: the nodes of
// the simplices of the regions that carry X.  A node on the interface of two
// materials carries one m per material, and the materials are not
// exchange-coupled across it (op_H_exch_X is assembled over X's simplices,
// nmag_lam.py:443-445,587-588).  The demagnetising potential lives on the
// nodes of the whole magnetic mesh and sees every material's charges.
//
// Layout.  The handle's mesh is the site mesh: the disjoint union of the
// materials' sub-meshes, sites numbered material by material (in the order
// given), mesh nodes ascending within a material.  Its assembly gives, block
// by block, each material's exchange operator K_X, box volumes and weak
// divergence D_X -- with the surface term on the faces where X ends, the
// reference's D/Dxj term (nmag_lam.py:446-451, fem.ml:5107-5150).  The
// potential mesh (all magnetic simplices) is held by an inner handle (pot)
// that owns the Poisson solves, the BEM and their precision forms.
//
// Per evaluation: rho_s = -Ms_X (D_X m_X)_s at the sites; rho_i = sum of the
// charges of node i's sites (node -> sites CSR, fixed order); the inner
// handle's pipeline gives phi on the nodes; then per site s of node i:
// H_demag = -(G phi)_i / V_i on the potential mesh, H_exch = -c_X (K_X m)_s /
// V_s, uniaxial anisotropy of X, H_total = ((H_ext + H_exch) + H_anis) +
// H_demag and the LLG equation with X's coefficients (nmag_lam.py:377-430).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "nmg_internal.h"

namespace nmg {
namespace {

inline unsigned nblk_s(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// rho_s = -Ms_X (D m)_s on the site mesh (D is block diagonal by material).
__global__ void k_div_sites(int S, int nnz, const SiteMat *__restrict__ mt, const int32_t *__restrict__ site_mat,
                            const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col_idx,
                            const double *__restrict__ D, const double *__restrict__ m, double *__restrict__ rho,
                            int nrep) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)S * nrep) return;
  const int b = (int)(g / S), s = (int)(g - (long long)b * S);
  const double *mb = m + (size_t)b * 3 * S;
  double acc = 0.0;
  for (int k = row_ptr[s]; k < row_ptr[s + 1]; ++k) {
    const double *mj = mb + 3 * (size_t)col_idx[k];
    acc += (D[k] * mj[0] + D[(size_t)nnz + k] * mj[1]) + D[2 * (size_t)nnz + k] * mj[2];
  }
  rho[g] = -(mt[site_mat[s]].Ms * acc);
}

// rho_i (potential mesh) = sum over the sites of node i, in site order.
__global__ void k_scatter_sites(int Np, const int32_t *__restrict__ node_ptr, const int32_t *__restrict__ node_sites,
                                const double *__restrict__ rho_s, double *__restrict__ rho_p, int S, int nrep) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)Np * nrep) return;
  const int b = (int)(g / Np), i = (int)(g - (long long)b * Np);
  double acc = 0.0;
  for (int k = node_ptr[i]; k < node_ptr[i + 1]; ++k) acc += rho_s[(size_t)b * S + node_sites[k]];
  rho_p[g] = acc;
}

// phi at the sites (the potential of each site's node), for the read-out.
__global__ void k_gather_sites(int S, const int32_t *__restrict__ site_node, const double *__restrict__ phi_p,
                               double *__restrict__ phi_s, int Np, int nrep) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)S * nrep) return;
  const int b = (int)(g / S), s = (int)(g - (long long)b * S);
  phi_s[g] = phi_p[(size_t)b * Np + site_node[s]];
}

struct SiteArgs {
  int S, nnz, Np, nnzp, nrep;
  const int32_t *row_ptr, *col_idx;           // site mesh
  const double *K, *ivol;
  const int32_t *prow, *pcol;                 // potential mesh
  const double *G, *pivol, *phi;
  const int32_t *site_node, *site_mat;
  const SiteMat *mt;
  const int32_t *node_ptr, *node_sites;       // node -> sites, for the local coupling
  const double *lc;                           // local coupling coefficients or null
  int n_mats;
  const double *m, *h_ext, *pin;
  double *h_exch, *h_demag, *h_anis, *h_total, *dmdt;
};

// H_lc of site s (material X at node i): sum over the node's other sites s'
// (material Y) of lc[X][Y] m_s' (nmag_lam.py:16-62, "have_m_Y" = node i
// carries a site of Y).
__device__ __forceinline__ void local_coupling(const SiteArgs &a, int s, int X, const double *mm, double *hl) {
  const int i = a.site_node[s];
  for (int k = a.node_ptr[i]; k < a.node_ptr[i + 1]; ++k) {
    const int s2 = a.node_sites[k];
    if (s2 == s) continue;
    const double c = a.lc[2 * (X * a.n_mats + a.site_mat[s2])];
    const double *m2 = mm + 3 * (size_t)s2;
    hl[0] += c * m2[0]; hl[1] += c * m2[1]; hl[2] += c * m2[2];
  }
}

__global__ void k_heff_llg_sites(SiteArgs a) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= (long long)a.S * a.nrep) return;
  const int b = (int)(g / a.S), s = (int)(g - (long long)b * a.S);
  const SiteMat c = a.mt[a.site_mat[s]];
  const double *mm = a.m + (size_t)b * 3 * a.S;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int k = a.row_ptr[s]; k < a.row_ptr[s + 1]; ++k) {
    const double *mj = mm + 3 * (size_t)a.col_idx[k];
    const double kv = a.K[k];
    s0 += kv * mj[0]; s1 += kv * mj[1]; s2 += kv * mj[2];
  }
  double hd[3] = {0.0, 0.0, 0.0};
  if (a.phi) {
    const int i = a.site_node[s];
    const double *ph = a.phi + (size_t)b * a.Np;
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int k = a.prow[i]; k < a.prow[i + 1]; ++k) {
      const double pj = ph[a.pcol[k]];
      g0 += a.G[k] * pj; g1 += a.G[(size_t)a.nnzp + k] * pj; g2 += a.G[2 * (size_t)a.nnzp + k] * pj;
    }
    const double piv = a.pivol[i];
    hd[0] = -g0 * piv; hd[1] = -g1 * piv; hd[2] = -g2 * piv;
  }
  const double ce = -c.c_exch * a.ivol[s];
  const double hx[3] = {ce * s0, ce * s1, ce * s2};
  const double *m = mm + 3 * (size_t)s;
  double ha[3] = {0.0, 0.0, 0.0};
  if (c.K1 != 0.0) {
    const double am = (c.ax * m[0] + c.ay * m[1]) + c.az * m[2];
    ha[0] = c.anis * am * (c.ax - am * m[0]);
    ha[1] = c.anis * am * (c.ay - am * m[1]);
    ha[2] = c.anis * am * (c.az - am * m[2]);
  }
  const double *he = a.h_ext + 3 * (size_t)g;
  double H[3];
  for (int d = 0; d < 3; ++d) H[d] = ((he[d] + hx[d]) + ha[d]) + hd[d];
  if (a.lc) {   // H_total = ... + H_lc (nmag_lam.py:404)
    double hl[3] = {0.0, 0.0, 0.0};
    local_coupling(a, s, a.site_mat[s], mm, hl);
    for (int d = 0; d < 3; ++d) H[d] += hl[d];
  }
  const double mxH[3] = {m[1] * H[2] - m[2] * H[1], m[2] * H[0] - m[0] * H[2], m[0] * H[1] - m[1] * H[0]};
  const double mxmxH[3] = {m[1] * mxH[2] - m[2] * mxH[1], m[2] * mxH[0] - m[0] * mxH[2],
                           m[0] * mxH[1] - m[1] * mxH[0]};
  const double c3 = c.C3 * (1.0 - ((m[0] * m[0] + m[1] * m[1]) + m[2] * m[2]));
  double f[3];
  for (int d = 0; d < 3; ++d) f[d] = (c.C1 * mxH[d] + c.C2 * mxmxH[d]) + c3 * m[d];
  if (a.pin) {
    const double p = a.pin[s];
    for (int d = 0; d < 3; ++d) f[d] *= p;
  }
  for (int d = 0; d < 3; ++d) {
    const size_t o = 3 * (size_t)g + d;
    a.h_exch[o] = hx[d]; a.h_demag[o] = hd[d]; a.h_anis[o] = ha[d]; a.h_total[o] = H[d];
    a.dmdt[o] = f[d];
  }
}

// Energy densities per site with the site's material (nmag_lam.py:454-460).
__global__ void k_energy_sites(long long SB, int S, const SiteMat *__restrict__ mt, const int32_t *__restrict__ site_mat,
                               const double *__restrict__ m, const double *__restrict__ hx,
                               const double *__restrict__ hd, const double *__restrict__ he, double *__restrict__ E,
                               const int32_t *__restrict__ site_node, const int32_t *__restrict__ node_ptr,
                               const int32_t *__restrict__ node_sites, const double *__restrict__ lc, int n_mats) {
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (g >= SB) return;
  const int s = (int)(g % S), X = site_mat[s];
  const SiteMat c = mt[X];
  const double *mi = m + 3 * (size_t)g, *x = hx + 3 * (size_t)g, *d = hd + 3 * (size_t)g, *e = he + 3 * (size_t)g;
  const double ex = c.E_half * ((mi[0] * x[0] + mi[1] * x[1]) + mi[2] * x[2]);
  const double dm = c.E_half * ((mi[0] * d[0] + mi[1] * d[1]) + mi[2] * d[2]);
  const double ez = c.E_ext * ((mi[0] * e[0] + mi[1] * e[1]) + mi[2] * e[2]);
  double an = 0.0;
  if (c.K1 != 0.0) {
    const double am = (c.ax * mi[0] + c.ay * mi[1]) + c.az * mi[2];
    an = -c.K1 * am * am;
  }
  double el = 0.0;   // E_lc = sum over the node's other sites of lc_e[X][Y] m_X . m_Y, added to E_total
  if (lc) {
    const double *mb = m + 3 * (size_t)(g - s);
    const int i = site_node[s];
    for (int k = node_ptr[i]; k < node_ptr[i + 1]; ++k) {
      const int s2 = node_sites[k];
      if (s2 == s) continue;
      const double *m2 = mb + 3 * (size_t)s2;
      el += lc[2 * (X * n_mats + site_mat[s2]) + 1] * ((mi[0] * m2[0] + mi[1] * m2[1]) + mi[2] * m2[2]);
    }
  }
  E[g] = ex; E[SB + g] = dm; E[2 * SB + g] = ez; E[3 * SB + g] = an;
  E[4 * SB + g] = (((dm + ex) + ez) + an) + el;
}

// Block partials over sites [s0, s0 + n) of member b: V, V m (3), V E_k (5).
__global__ void k_site_avg(int n, int s0, const double *__restrict__ m, const double *__restrict__ vol,
                           const double *__restrict__ E, size_t estride, double *__restrict__ part) {
  __shared__ double sm[32][9];
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int s = s0 + j;
    const double V = vol[s];
    v[0] += V;
    for (int d = 0; d < 3; ++d) v[1 + d] += V * m[3 * (size_t)s + d];
    if (E) for (int k = 0; k < 5; ++k) v[4 + k] += V * E[(size_t)k * estride + s];
  }
  for (int k = 0; k < 9; ++k)
    for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) for (int k = 0; k < 9; ++k) sm[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 9) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sm[q][threadIdx.x];
    part[9 * blockIdx.x + threadIdx.x] = t;
  }
}

SiteMat site_mat_of(const nmg_material &x) {
  SiteMat c;
  c.Ms = x.Ms; c.c_exch = x.exch_coeff; c.C1 = x.C1; c.C2 = x.C2; c.C3 = x.C3; c.K1 = x.K1;
  c.ax = x.axis[0]; c.ay = x.axis[1]; c.az = x.axis[2]; c.anis = x.anis_coeff;
  c.E_half = x.E_coeff_half; c.E_ext = x.E_coeff_ext;
  return c;
}

}  // namespace

int rhs_eval_sites(nmg_handle *h, const double *d_m, double *d_dmdt) {
  Mesh &M = h->mesh;
  Workspace &W = h->ws;
  nmg_handle *P = h->pot;
  cudaStream_t st = h->stream;
  const int S = M.N, B = h->nrep;
  const long long SB = (long long)S * B;
  const bool demag = h->opt.do_demag && P->mesh.nb > 0;
  if (demag) {
    k_div_sites<<<nblk_s(SB, 256), 256, 0, st>>>(S, M.nnz, h->sites.mtab, h->sites.site_mat, M.row_ptr, M.col_idx,
                                                  M.D, d_m, W.rho, B);
    k_scatter_sites<<<nblk_s((long long)P->mesh.N * B, 256), 256, 0, st>>>(
        P->mesh.N, h->sites.node_ptr, h->sites.node_sites, W.rho, P->ws.rho, S, B);
    h->launches += 2;
    if (demag_from_rho(P)) {
      h->last_error = P->last_error;
      return 100;
    }
    h->launches += P->launches;
    P->launches = 0;
    k_gather_sites<<<nblk_s(SB, 256), 256, 0, st>>>(S, h->sites.site_node, P->ws.phi, W.phi, P->mesh.N, B);
    ++h->launches;
  }
  SiteArgs a;
  a.S = S; a.nnz = M.nnz; a.Np = P->mesh.N; a.nnzp = P->mesh.nnz; a.nrep = B;
  a.row_ptr = M.row_ptr; a.col_idx = M.col_idx; a.K = M.K; a.ivol = M.ivol;
  a.prow = P->mesh.row_ptr; a.pcol = P->mesh.col_idx; a.G = P->mesh.G; a.pivol = P->mesh.ivol;
  a.phi = demag ? P->ws.phi.p : nullptr;
  a.site_node = h->sites.site_node; a.site_mat = h->sites.site_mat; a.mt = h->sites.mtab;
  a.node_ptr = h->sites.node_ptr; a.node_sites = h->sites.node_sites; a.lc = h->sites.lc.p;
  a.n_mats = h->sites.n_mats;
  a.m = d_m; a.h_ext = W.h_ext; a.pin = h->pin.p;
  a.h_exch = W.h_exch; a.h_demag = W.h_demag; a.h_anis = W.h_anis; a.h_total = W.h_total;
  a.dmdt = d_dmdt ? d_dmdt : W.dmdt.p;
  {
    NMG_PROF_BEGIN(h, 3);
    k_heff_llg_sites<<<nblk_s(SB, 128), 128, 0, st>>>(a);
    ++h->launches;
    NMG_PROF_END(h);
  }
  h->n_rhs++;
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

// The demag response of a site direction v: its charges per site, summed onto
// the potential mesh's nodes, through the potential handle's pipeline on the
// Jacobian's own buffers; hdv per node of the potential mesh.
int demag_response_sites(nmg_handle *h, const double *d_v) {
  Mesh &M = h->mesh;
  nmg_handle *P = h->pot;
  JacDemag &J = h->jd;
  if (jac_prepare(P, J)) {
    h->last_error = "exact Jacobian: cannot allocate the demag response buffers";
    return 100;
  }
  const int S = M.N, B = h->nrep;
  cudaStream_t st = h->stream;
  k_div_sites<<<nblk_s((long long)S * B, 256), 256, 0, st>>>(S, M.nnz, h->sites.mtab, h->sites.site_mat, M.row_ptr,
                                                              M.col_idx, M.D, d_v, h->ws.rho, B);
  k_scatter_sites<<<nblk_s((long long)P->mesh.N * B, 256), 256, 0, st>>>(P->mesh.N, h->sites.node_ptr,
                                                                          h->sites.node_sites, h->ws.rho, J.rho, S, B);
  h->launches += 2;
  const int rc = jac_demag_solve(P, J, h->jac_rtol);
  h->launches += P->launches;
  P->launches = 0;
  if (rc) h->last_error = P->last_error.empty() ? "exact Jacobian: demag response failed" : P->last_error;
  return rc;
}

int energy_density_sites(nmg_handle *h, const double *d_m, double *d_E5) {
  Workspace &W = h->ws;
  const long long SB = (long long)h->mesh.N * h->nrep;
  k_energy_sites<<<nblk_s(SB, 256), 256, 0, h->stream>>>(SB, h->mesh.N, h->sites.mtab, h->sites.site_mat, d_m,
                                                          W.h_exch, W.h_demag, W.h_ext, d_E5, h->sites.site_node,
                                                          h->sites.node_ptr, h->sites.node_sites, h->sites.lc.p,
                                                          h->sites.n_mats);
  ++h->launches;
  return cudaGetLastError() == cudaSuccess ? 0 : 100;
}

}  // namespace nmg

namespace {

std::string g_sites_error;

int sites_fail(int code, const std::string &msg) {
  nmg::set_handleless_error(msg);
  return code;
}

}  // namespace

extern "C" {

int nmg_create_materials(const double *coords, int n_nodes, const int32_t *tets, int n_tets, const int32_t *tet_region,
                         int n_regions, const int32_t *region_ptr, const int32_t *region_mats,
                         const nmg_material *mats, int n_mats, const nmg_options *opt, nmg_handle **out) {
  if (!coords || !tets || !tet_region || !region_ptr || !region_mats || !mats || !out)
    return sites_fail(-1, "nmg_create_materials: NULL input array");
  if (n_nodes < 4 || n_tets < 1 || n_regions < 1 || n_mats < 1)
    return sites_fail(-2, "nmg_create_materials: need nodes, tetrahedra, regions and materials");
  if (region_ptr[0] != 0) return sites_fail(-2, "nmg_create_materials: region_ptr[0] must be 0");
  for (int r = 0; r < n_regions; ++r)
    if (region_ptr[r + 1] < region_ptr[r]) return sites_fail(-2, "nmg_create_materials: region_ptr not ascending");
  for (int k = 0; k < region_ptr[n_regions]; ++k)
    if (region_mats[k] < 0 || region_mats[k] >= n_mats)
      return sites_fail(-2, "nmg_create_materials: region names a missing material");
  for (long long t = 0; t < n_tets; ++t)
    if (tet_region[t] < 1 || tet_region[t] > n_regions)
      return sites_fail(-3, "nmg_create_materials: tetrahedron with a region outside 1..n_regions");
  for (long long k = 0; k < 4LL * n_tets; ++k)
    if (tets[k] < 0 || tets[k] >= n_nodes) return sites_fail(-3, "nmg_create_materials: tetrahedron refers to a missing node");
  nmg_options o{};
  if (opt) o = *opt;
  else {
    o.do_demag = 1;
    o.nbc_rtol = o.dbc_rtol = 1e-5;
    o.nbc_atol = o.dbc_atol = 1e-50;
    o.nbc_maxits = o.dbc_maxits = 10000;
  }
  // sites: per material the tetrahedra of its regions, their nodes ascending
  std::vector<std::vector<char>> region_has(n_mats, std::vector<char>(n_regions + 1, 0));
  for (int r = 0; r < n_regions; ++r)
    for (int k = region_ptr[r]; k < region_ptr[r + 1]; ++k) region_has[region_mats[k]][r + 1] = 1;
  std::vector<int32_t> site_node, site_mat, site_tets;
  std::vector<int> offset(n_mats), count(n_mats);
  std::vector<int32_t> local(n_nodes);
  for (int x = 0; x < n_mats; ++x) {
    std::vector<char> used(n_nodes, 0);
    std::vector<int> mt;
    for (int t = 0; t < n_tets; ++t)
      if (region_has[x][tet_region[t]]) {
        mt.push_back(t);
        for (int c = 0; c < 4; ++c) used[tets[4 * (size_t)t + c]] = 1;
      }
    offset[x] = (int)site_node.size();
    for (int i = 0; i < n_nodes; ++i)
      if (used[i]) {
        local[i] = (int32_t)site_node.size();
        site_node.push_back(i);
        site_mat.push_back(x);
      }
    count[x] = (int)site_node.size() - offset[x];
    for (int t : mt)
      for (int c = 0; c < 4; ++c) site_tets.push_back(local[tets[4 * (size_t)t + c]]);
    if (count[x] == 0) return sites_fail(-2, "nmg_create_materials: material " + std::to_string(x) + " has no simplices");
  }
  const int S = (int)site_node.size();
  // the site mesh's coordinates, and the magnetic mesh's simplices (every region)
  std::vector<double> scoords(3 * (size_t)S);
  for (int s = 0; s < S; ++s)
    for (int d = 0; d < 3; ++d) scoords[3 * (size_t)s + d] = coords[3 * (size_t)site_node[s] + d];
  // node -> sites (sites ascending)
  std::vector<int32_t> node_ptr(n_nodes + 1, 0), node_sites(S);
  for (int s = 0; s < S; ++s) node_ptr[site_node[s] + 1]++;
  for (int i = 0; i < n_nodes; ++i) node_ptr[i + 1] += node_ptr[i];
  {
    std::vector<int32_t> fill(node_ptr.begin(), node_ptr.end() - 1);
    for (int s = 0; s < S; ++s) node_sites[fill[site_node[s]]++] = s;
  }
  for (int i = 0; i < n_nodes; ++i)
    if (node_ptr[i + 1] == node_ptr[i]) return sites_fail(-3, "nmg_create_materials: a node outside every tetrahedron");
  // the potential mesh: all magnetic simplices, with the demag pipeline
  nmg_handle *P = nullptr;
  nmg_options po = o;
  int rc = nmg_create(coords, n_nodes, tets, n_tets, &mats[0], &po, &P);
  if (rc) return rc;
  // the site mesh: no demag pipeline of its own (the potential mesh's serves it)
  nmg_options so = o;
  so.do_demag = 0;
  so.bem_precision = 0;
  so.bem_anchor_tol = 0.0;
  nmg_handle *H = nullptr;
  rc = nmg_create(scoords.data(), S, site_tets.data(), (int)(site_tets.size() / 4), &mats[0], &so, &H);
  if (rc) {
    nmg_destroy(P);
    return rc;
  }
  H->opt.do_demag = o.do_demag;
  H->pot = P;
  // one stream for both: the site handle's work and the potential's are ordered
  cudaStreamSynchronize(H->stream);
  cudaStreamDestroy(H->stream);
  H->stream = P->stream;
  H->own_stream = false;
  nmg::Sites &St = H->sites;
  St.n_mats = n_mats;
  St.offset = offset;
  St.count = count;
  std::vector<nmg::SiteMat> tab(n_mats);
  for (int x = 0; x < n_mats; ++x) tab[x] = nmg::site_mat_of(mats[x]);
  bool ok = St.site_node.alloc(S) == cudaSuccess && St.site_mat.alloc(S) == cudaSuccess &&
            St.node_ptr.alloc(n_nodes + 1) == cudaSuccess && St.node_sites.alloc(S) == cudaSuccess &&
            St.mtab.alloc(n_mats) == cudaSuccess;
  ok = ok && cudaMemcpy(St.site_node.p, site_node.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(St.site_mat.p, site_mat.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(St.node_ptr.p, node_ptr.data(), sizeof(int32_t) * (n_nodes + 1), cudaMemcpyHostToDevice) ==
           cudaSuccess &&
       cudaMemcpy(St.node_sites.p, node_sites.data(), sizeof(int32_t) * S, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(St.mtab.p, tab.data(), sizeof(nmg::SiteMat) * n_mats, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    nmg_destroy(H);
    return sites_fail(100, "nmg_create_materials: device set-up failed");
  }
  *out = H;
  return 0;
}

int nmg_set_site_material(nmg_handle *h, int material, const nmg_material *mat) {
  if (!h || !mat) return -1;
  if (!h->pot) return -2;
  if (material < 0 || material >= h->sites.n_mats) return -2;
  const nmg::SiteMat c = nmg::site_mat_of(*mat);
  if (cudaMemcpyAsync(h->sites.mtab.p + material, &c, sizeof(c), cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return 100;
  if (material == 0) h->mat = *mat;
  h->ts_ready = 0;
  return 0;
}

int nmg_set_local_coupling(nmg_handle *h, int mat1, int mat2, double h_coeff, double e_coeff) {
  if (!h) return -1;
  if (!h->pot) return -2;
  const int n = h->sites.n_mats;
  if (mat1 < 0 || mat1 >= n || mat2 < 0 || mat2 >= n || mat1 == mat2) return -2;
  if (!std::isfinite(h_coeff) || !std::isfinite(e_coeff)) return -5;
  nmg::Sites &St = h->sites;
  if (St.lc_host.empty()) St.lc_host.assign(2 * (size_t)n * n, 0.0);
  St.lc_host[2 * ((size_t)mat1 * n + mat2)] = h_coeff;
  St.lc_host[2 * ((size_t)mat1 * n + mat2) + 1] = e_coeff;
  if (!St.lc.p && St.lc.alloc(St.lc_host.size()) != cudaSuccess) return 100;
  if (cudaMemcpyAsync(St.lc.p, St.lc_host.data(), sizeof(double) * St.lc_host.size(), cudaMemcpyHostToDevice,
                      h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return 100;
  h->ts_ready = 0;
  return 0;
}

int nmg_site_info(const nmg_handle *h, int32_t *site_node, int32_t *site_material) {
  if (!h) return -1;
  if (!h->pot) return -2;
  const size_t S = h->mesh.N;
  if (site_node && cudaMemcpy(site_node, h->sites.site_node.p, sizeof(int32_t) * S, cudaMemcpyDeviceToHost))
    return 100;
  if (site_material && cudaMemcpy(site_material, h->sites.site_mat.p, sizeof(int32_t) * S, cudaMemcpyDeviceToHost))
    return 100;
  return 0;
}

int nmg_material_averages(nmg_handle *h, int material, int member, double avg_m[3], double energies[5]) {
  if (!h || !avg_m) return -1;
  const int S = h->mesh.N;
  int s0 = 0, n = S;
  if (h->pot) {
    if (material < 0 || material >= h->sites.n_mats) return -2;
    s0 = h->sites.offset[material];
    n = h->sites.count[material];
  } else if (material != 0) {
    return -2;
  }
  if (member < 0 || member >= h->nrep) return -2;
  const double *m = h->ws.m.p + (size_t)member * 3 * S;
  const double *E = nullptr;
  if (energies) {
    if (nmg::energy_density(h, h->ws.m, h->ws.E5)) return 100;
    E = h->ws.E5.p + (size_t)member * S;
  }
  const int blocks = 64;
  nmg::DevBuf<double> part;
  if (part.alloc(9 * blocks) != cudaSuccess) return 100;
  nmg::k_site_avg<<<blocks, 256, 0, h->stream>>>(n, s0, m, h->mesh.vol, E, (size_t)S * h->nrep, part.p);
  ++h->launches;
  std::vector<double> hp(9 * blocks);
  if (cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * 9 * blocks, cudaMemcpyDeviceToHost, h->stream) ||
      cudaStreamSynchronize(h->stream))
    return 100;
  double tot[9] = {0};
  for (int b = 0; b < blocks; ++b)
    for (int j = 0; j < 9; ++j) tot[j] += hp[9 * b + j];
  for (int d = 0; d < 3; ++d) avg_m[d] = tot[1 + d] / tot[0];
  if (energies) for (int k = 0; k < 5; ++k) energies[k] = tot[4 + k];
  return 0;
}

}  // extern "C"
