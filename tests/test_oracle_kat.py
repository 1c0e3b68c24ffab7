"""Known-answer pins of the CPU oracle (runs on CPU).

The reference as a whole cannot run here and ships no golden vectors (its
plain-C BEM stub is compiled and pins the BEM fill: test_oracle_ref.py);
these tests pin the rest of the oracle against facts that hold for the
reference's method: closed-form mesh counts, the BEM row-sum identity,
Lindholm weights against quadrature, the exchange field of a uniform state,
the cube's demagnetising factor and the analytic single-spin LLG solution.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle
from conftest import permalloy, seeded_m

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


@pytest.fixture(scope="module")
def ocube(cube):
    return oracle.OracleMesh(cube.points, cube.simplices)


def test_cube_counts_match_closed_form(ocube):
    g = GOLD["cube_10"]
    assert ocube.n_nodes == g["nodes"] and ocube.n_tets == g["tets"]
    assert ocube.nnz == g["nnz"]
    assert ocube.nb == g["boundary_nodes"]
    assert int((ocube.nbr < 0).sum()) == g["outer_faces"]


def test_small_box_counts(small_box):
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    g = GOLD["box_4x3x2"]
    assert (om.n_nodes, om.nnz, om.nb, int((om.nbr < 0).sum())) == (g["nodes"], g["nnz"], g["boundary_nodes"],
                                                                      g["outer_faces"])


def test_csr_is_symmetric_pattern_and_sorted(ocube):
    rp, ci = ocube.row_ptr, ocube.col_idx
    for i in range(ocube.n_nodes):
        row = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) > 0)
        assert i in row
    import scipy.sparse as sp
    K = sp.csr_matrix((ocube.K, ci, rp))
    assert abs(K - K.T).max() < 1e-12
    assert np.abs(K @ np.ones(ocube.n_nodes)).max() < 1e-12   # constants in the kernel


def test_volumes_and_gradient_identities(ocube, cube):
    assert abs(ocube.vol.sum() - 27000.0) < 1e-9
    import scipy.sparse as sp
    x = cube.points
    for d in range(3):
        G = sp.csr_matrix((ocube.G[d], ocube.col_idx, ocube.row_ptr))
        # int phi_i d_d(x_d) = V_i for a linear field
        assert np.allclose(G @ x[:, d], ocube.vol, rtol=1e-12, atol=1e-12)
        D = sp.csr_matrix((ocube.D[d], ocube.col_idx, ocube.row_ptr))
        # divergence theorem: column sums of the full div operator vanish
        assert np.abs(np.ones(ocube.n_nodes) @ D).max() < 1e-10


def test_bem_row_sums_are_minus_one(ocube):
    # constant double-layer density on a closed surface: sum_j B_ij = -1
    s = ocube.bem.sum(axis=1)
    assert np.abs(s + 1.0).max() < 1e-9


def test_duplicate_interior_triangles_cancel(ocube):
    # the reference's node-based surface rule emits interior faces whose three
    # vertices are boundary nodes, once per side with opposite normals
    assert ocube.ntri > GOLD["cube_10"]["outer_faces"]
    assert (ocube.ntri - GOLD["cube_10"]["outer_faces"]) % 2 == 0


def test_lindholm_matches_quadrature_far_field():
    p0, p1, p2 = np.array([0.0, 0.0, 0.0]), np.array([2.0, 0.0, 0.0]), np.array([0.3, 1.7, 0.0])
    n = np.array([0.0, 0.0, 1.0])
    rng = np.random.default_rng(5)
    # Dunavant-like dense barycentric grid quadrature of
    # w_i = (1/4pi) int L_i d/dn_y (1/|x - y|) dA = (1/4pi) int L_i (x - y).n / |x - y|^3 dA
    # collapsed (Duffy) Gauss-Legendre rule on the triangle: u = a(1-b), v = a b
    g, w = np.polynomial.legendre.leggauss(40)
    a, b = np.meshgrid((g + 1) / 2, (g + 1) / 2, indexing="ij")
    wa, wb = np.meshgrid(w / 2, w / 2, indexing="ij")
    u, v = (a * (1 - b)).ravel(), (a * b).ravel()
    area = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0))
    wq = (wa * wb * a).ravel() * 2.0 * area
    y = p0[None] + u[:, None] * (p1 - p0)[None] + v[:, None] * (p2 - p0)[None]
    L = np.stack([1 - u - v, u, v])
    for _ in range(5):
        x = rng.normal(size=3) * 6.0 + np.array([0.5, 0.5, 0.0])
        x[2] = abs(x[2]) + 4.0 if rng.random() < 0.5 else -(abs(x[2]) + 4.0)
        r = y - x[None]
        kern = -(r @ n) / np.linalg.norm(r, axis=1) ** 3
        quad = (L * (kern * wq)[None]).sum(1) / (4 * math.pi)
        lh = oracle.lindholm_single(p0, p1, p2, n, x)
        assert np.allclose(lh, quad, rtol=1e-9, atol=1e-15), (lh, quad)


def test_solid_angle_of_octant():
    # the three unit vectors span one octant: 4 pi / 8
    a = oracle.solid_angle([0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1])
    assert abs(a - math.pi / 2) < 1e-14


def coeffs_of(mat):
    return mat.coefficients("nmag")


def test_su_coefficients_match_reference_formulas():
    g = GOLD["permalloy_alpha05"]
    c = permalloy(0.5).coefficients(None)
    assert math.isclose(c["Ms"], g["su_Ms"], rel_tol=1e-15)
    assert math.isclose(c["exch_coeff"], g["exch_prefactor"], rel_tol=1e-14)
    assert math.isclose(c["C1"], g["C1"], rel_tol=1e-14)
    assert math.isclose(c["C2"], g["C2"], rel_tol=1e-14)
    q = permalloy(0.5).coefficients("nmag")
    assert q["C1"] == -0.17688 and q["exch_coeff"] == 24.0583053511


def test_exchange_of_uniform_state_is_zero(ocube):
    s = oracle.OracleSim(ocube, coeffs_of(permalloy()), do_demag=False)
    m = np.tile([0.6, 0.0, 0.8], (ocube.n_nodes, 1))
    s.rhs(m)
    assert np.abs(s.field("H_exch")).max() < 1e-12


def test_exchange_of_quadratic_state_is_the_laplacian():
    """H_exch = exch_coeff * Laplacian(m) (the operator ($negJ$) <d/dxj H_exch||d/dxj m>
    with negJ = -su_exch_prefactor, nmag_lam.py:256,445): on the
    Kuhn-split box the P1 stiffness matrix is the 7-point stencil and the
    box volumes the cell volume, so at interior nodes the discrete Laplacian
    of a quadratic is exact -- on unequal spacings too."""
    from nmag import mesh
    msh = mesh.box_mesh(6, 5, 4, 2.0, 2.5, 1.5)
    om = oracle.OracleMesh(msh.points, msh.simplices, fill_bem=False)
    c = coeffs_of(permalloy())
    s = oracle.OracleSim(om, c, do_demag=False)
    p = msh.points
    m = np.stack([p[:, 0] ** 2, p[:, 1] ** 2 + 0.5 * p[:, 2], p[:, 0] * p[:, 1] - p[:, 2] ** 2], axis=1)
    s.rhs(m)
    H = s.field("H_exch")
    inner = np.all((p > p.min(0) + 1e-9) & (p < p.max(0) - 1e-9), axis=1)
    assert inner.sum() == 5 * 4 * 3
    assert np.abs(H[inner] / c["exch_coeff"] - np.array([2.0, 2.0, -2.0])).max() < 1e-12


def test_cube_demag_factor_is_one_third(ocube):
    s = oracle.OracleSim(ocube, coeffs_of(permalloy()), nbc=(1e-10, 1e-50, 5000), dbc=(1e-10, 1e-50, 5000))
    m = np.tile([1.0, 0.0, 0.0], (ocube.n_nodes, 1))
    s.rhs(m)
    H = s.field("H_demag")
    V = ocube.vol
    avg = (H * V[:, None]).sum(0) / V.sum() / 0.86
    assert abs(avg[0] + 1.0 / 3.0) < 0.01          # FEM/BEM on 10^3 cells: ~0.329
    assert abs(avg[1]) < 1e-9 and abs(avg[2]) < 1e-9


def analytic_spin(t, m0, C1, C2, H):
    """Exact solution of dm/dt = C1 m x H z + C2 m x (m x H z), |m| = 1."""
    mz0 = m0[2]
    phi0 = math.atan2(m0[1], m0[0])
    mz = np.tanh(-C2 * H * t + np.arctanh(mz0))
    phi = phi0 - C1 * H * t
    rho = np.sqrt(1 - mz ** 2)
    return np.stack([rho * np.cos(phi), rho * np.sin(phi), mz], axis=-1)


def test_bdf_single_spin_matches_analytic(small_box):
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    c = coeffs_of(permalloy(0.1))
    s = oracle.OracleSim(om, c, do_demag=False)
    H = 0.5
    s.set_h_ext([0.0, 0.0, H])
    m0 = np.array([math.sin(1.0), 0.0, math.cos(1.0)])
    s.ts_init(np.tile(m0, (om.n_nodes, 1)), rtol=1e-8, atol=1e-8)
    for t in (5.0, 20.0, 40.0):
        tr, m = s.ts_advance(t)
        ref = analytic_spin(t, m0, c["C1"], c["C2"], H)
        assert abs(tr - t) < 1e-12
        assert np.abs(m - ref[None]).max() < 2e-5, (t, np.abs(m - ref[None]).max())


def test_bdf_energy_decreases_with_damping(ocube):
    s = oracle.OracleSim(ocube, coeffs_of(permalloy(0.5)), nbc=(1e-8, 1e-50, 5000), dbc=(1e-8, 1e-50, 5000))
    m0 = seeded_m(ocube.n_nodes, seed=0, noise=0.3)
    s.ts_init(m0)
    E_prev = None
    for t in (1.0, 2.0, 4.0, 8.0):
        _, m = s.ts_advance(t)
        s.rhs(m)
        E = (s.energy_density(m)[4] * ocube.vol).sum()
        if E_prev is not None:
            assert E <= E_prev + 1e-9
        E_prev = E
        assert np.abs(np.linalg.norm(m, axis=1) - 1.0).max() < 1e-4
