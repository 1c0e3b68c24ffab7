"""Oracle for several magnetic materials (test infrastructure: only tests
import it).  CPU restatement of the reference's multi-material right-hand
side (interface/nmag/nmag_lam.py:183-470, 587-606, 734-832):

* every material X has its own m_X on its sites (the nodes of the simplices
  of its regions); its exchange operator op_H_exch_X and box volumes are
  assembled over X's simplices only (nmag_lam.py:443-445,587-588), so the
  sub-mesh of X (its sites, its simplices renumbered) gives them;
* op_div_m sums the materials: rho_i = -sum_X Ms_X (D_X m_X) at the site of
  node i in X, D_X the weak divergence over X's simplices with the surface
  term on the faces where X ends (nmag_lam.py:446-451; fem.ml:5107-5150) --
  the outer faces of X's sub-mesh;
* phi (Neumann solve, BEM, Dirichlet solve) and H_demag = -G phi / V live on
  the nodes of the whole magnetic mesh (nmag_lam.py:591-606,740-760);
* H_total_X = H_ext + H_exch_X + H_anis_X + H_demag at X's sites and the LLG
  equation with X's coefficients (nmag_lam.py:377-430).

The meshes' operators and BEM come from the C oracle (oracle.OracleMesh);
the Poisson problems are solved directly (scipy), so the result is exact up
to rounding.  Parity is pinned against the single-material C oracle (one
material; materials on disjoint regions) and by known answers (cancelling
interface charges, zero total charge, no exchange across an interface).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle


def _csr(om, vals):
    return sp.csr_matrix((vals, om.col_idx, om.row_ptr), shape=(om.n_nodes, om.n_nodes))


class MultiOracle(object):
    """points (N,3), simplices (T,4), regions (T,) >= 1 of the magnetic mesh;
    layer: nmag.sites.SiteLayer of it; coeffs: material name ->
    MagMaterial.coefficients() (Ms, exch_coeff, C1..C5, K1/axis/anis_coeff,
    anis_poly)."""

    def __init__(self, points, simplices, layer, coeffs):
        self.layer = layer
        self.coeffs = coeffs
        self.pm = oracle.OracleMesh(points, simplices, fill_bem=True)
        pm = self.pm
        self.N = pm.n_nodes
        self.K = _csr(pm, pm.K)
        self.G = [_csr(pm, pm.G[d]) for d in range(3)]
        # Neumann: K phi = rho with sum(phi) = 0 (the constant null space)
        one = np.ones((self.N, 1))
        self._neu = spla.splu(sp.bmat([[self.K, sp.csr_matrix(one)], [sp.csr_matrix(one.T), None]]).tocsc())
        # Dirichlet: interior rows of K, boundary values given
        self.bnd = pm.node_of_b.astype(np.int64)
        inner = np.setdiff1d(np.arange(self.N), self.bnd)
        self.inner = inner
        self._dir = spla.splu(self.K[inner][:, inner].tocsc())
        self._kib = self.K[inner][:, self.bnd]
        self.sub = {}
        for name in layer.materials:
            p, t = layer.submesh(name, points)
            om = oracle.OracleMesh(p, t, fill_bem=False)
            self.sub[name] = (om, _csr(om, om.K), [_csr(om, om.D[d]) for d in range(3)])
        self.h_ext = np.zeros((self.N, 3))
        self.local_couplings = {}

    def set_local_coupling(self, name1, name2, h_coeff, e_coeff):
        """H_lc of name1 gains h_coeff m_name2 at the nodes carrying both
        (nmag_lam.py:16-62); its energy density e_coeff m_name1 . m_name2."""
        self.local_couplings[(name1, name2)] = (h_coeff, e_coeff)

    def set_h_ext(self, h):
        self.h_ext = np.broadcast_to(np.asarray(h, dtype=np.float64), (self.N, 3)).copy()

    def _anis(self, c, m):
        H = np.zeros_like(m)
        if c.get("K1", 0.0) != 0.0:
            a = np.asarray(c["axis"], dtype=np.float64)
            am = m @ a
            H += c["anis_coeff"] * am[:, None] * (a[None, :] - am[:, None] * m)
        poly = c.get("anis_poly")
        if poly is not None:
            hp, hc = poly[2], np.reshape(poly[3], (-1, 3))
            for p, cf in zip(hp, hc):
                mono = m[:, 0] ** (p & 15) * m[:, 1] ** ((p >> 4) & 15) * m[:, 2] ** ((p >> 8) & 15)
                H += np.outer(mono, cf)
        return H

    def rhs(self, m_sites):
        """dm/dt (S,3) for m of every material's sites (S,3, material-major);
        the fields of the evaluation in self.fields."""
        L = self.layer
        m = np.asarray(m_sites, dtype=np.float64).reshape(L.n_sites, 3)
        # charges: -Ms_X D_X m_X at X's sites, summed onto the nodes
        rho_s = np.zeros(L.n_sites)
        for name in L.materials:
            om, K, D = self.sub[name]
            s = L.sites_of(name)
            mx = m[s]
            rho_s[s] = -self.coeffs[name]["Ms"] * ((D[0] @ mx[:, 0] + D[1] @ mx[:, 1]) + D[2] @ mx[:, 2])
        rho = L.scatter(rho_s)
        phi1 = self._neu.solve(np.concatenate([rho - rho.mean(), [0.0]]))[:self.N]
        phi2b = self.pm.bem @ phi1[self.bnd]
        phi2 = np.zeros(self.N)
        phi2[self.bnd] = phi2b
        phi2[self.inner] = self._dir.solve(-(self._kib @ phi2b))
        phi = phi1 + phi2
        hd = -np.stack([self.G[d] @ phi for d in range(3)], axis=1) / self.pm.vol[:, None]
        H_exch = np.zeros_like(m)
        H_anis = np.zeros_like(m)
        for name in L.materials:
            om, K, D = self.sub[name]
            s = L.sites_of(name)
            c = self.coeffs[name]
            H_exch[s] = -c["exch_coeff"] * (K @ m[s]) / om.vol[:, None]
            H_anis[s] = self._anis(c, m[s])
        H_total = ((L.gather(self.h_ext) + H_exch) + H_anis) + L.gather(hd)
        # local couplings: at every node, each site's H_lc from the node's other sites
        H_lc = np.zeros_like(m)
        E_lc = np.zeros(L.n_sites)
        if self.local_couplings:
            names = L.materials
            for i in range(self.N):
                sites = L.node_site_idx[L.node_site_ptr[i]:L.node_site_ptr[i + 1]]
                for s1 in sites:
                    for s2 in sites:
                        if s1 == s2:
                            continue
                        c = self.local_couplings.get((names[L.site_material[s1]], names[L.site_material[s2]]))
                        if c is not None:
                            H_lc[s1] += c[0] * m[s2]
                            E_lc[s1] += c[1] * float(m[s1] @ m[s2])
            H_total = H_total + H_lc
        dmdt = np.zeros_like(m)
        for name in L.materials:
            s = L.sites_of(name)
            c = self.coeffs[name]
            ms, H = m[s], H_total[s]
            mxH = np.cross(ms, H)
            dmdt[s] = (c["C1"] * mxH + c["C2"] * np.cross(ms, mxH)) + (c["C3"] * (1.0 - np.sum(ms * ms, 1)))[:, None] * ms
        self.fields = {"rho": rho, "rho_sites": rho_s, "phi": phi, "H_demag": hd, "H_exch": H_exch,
                       "H_anis": H_anis, "H_total": H_total, "dmdt": dmdt, "H_lc": H_lc, "E_lc": E_lc}
        return dmdt
