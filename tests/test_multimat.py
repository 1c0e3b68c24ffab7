"""Several magnetic materials: the site layer (nmag.sites) and the oracle's
multi-material right-hand side (oracle/multimat.py), pinned against the
single-material C oracle and by known answers.  CPU only."""
import numpy as np
import pytest

import nmag
from nmag import SI
from nmag.mesh import Mesh, box_mesh
from nmag.sites import SiteLayer
from conftest import seeded_m

TIGHT = (1e-13, 1e-50, 20000)


def halves():
    """A 12 x 6 x 4 nm box split at x = 6 nm into regions 1 and 2."""
    b = box_mesh(6, 3, 2, 2.0)
    cx = b.points[b.simplices].mean(1)[:, 0]
    return Mesh(b.points, b.simplices, np.where(cx < 6.0, 1, 2))


def two_boxes():
    """Two 6 x 6 x 4 nm boxes 4 nm apart (regions 1 and 2)."""
    a = box_mesh(3, 3, 2, 2.0)
    b = box_mesh(3, 3, 2, 2.0, origin=(10.0, 0.0, 0.0))
    pts = np.concatenate([a.points, b.points])
    sim = np.concatenate([a.simplices, b.simplices + a.n_nodes])
    reg = np.concatenate([np.ones(a.n_tets, np.int32), np.full(b.n_tets, 2, np.int32)])
    return Mesh(pts, sim, reg)


def material(name, Ms=8.6e5, A=1.3e-11, alpha=0.3):
    return nmag.MagMaterial(name, Ms=SI(Ms, "A/m"), exchange_coupling=SI(A, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(2.211e5, "m/A s"))


def test_site_layer():
    msh = halves()
    L = SiteLayer(msh, [["A"], ["B"]])
    assert L.materials == ["A", "B"]
    x = msh.points[:, 0]
    nA, nB = L.nodes
    assert np.array_equal(nA, np.nonzero(x <= 6.0)[0]) and np.array_equal(nB, np.nonzero(x >= 6.0)[0])
    assert L.n_sites == len(nA) + len(nB) == msh.n_nodes + np.sum(x == 6.0)
    # interface nodes have two sites, A's first
    k = int(np.nonzero(x == 6.0)[0][0])
    sites = L.node_site_idx[L.node_site_ptr[k]:L.node_site_ptr[k + 1]]
    assert [L.site_material[s] for s in sites] == [0, 1] and all(L.site_node[s] == k for s in sites)
    p, t = L.submesh("B", msh.points)
    assert np.allclose(p[t], msh.points[msh.simplices[L.tets[1]]])
    v = np.arange(L.n_sites, dtype=float)
    assert np.allclose(L.scatter(v)[k], sites.sum())
    assert np.array_equal(L.gather(np.arange(msh.n_nodes)), L.site_node)
    # a region with two materials gives both of them its nodes
    L2 = SiteLayer(msh, [["A", "B"], ["B"]])
    assert len(L2.nodes[0]) == len(nA) and len(L2.nodes[1]) == msh.n_nodes


def _single_oracle(msh, mat, h):
    import oracle
    om = oracle.OracleMesh(msh.points, msh.simplices)
    s = oracle.OracleSim(om, mat.coefficients("nmag"), nbc=TIGHT, dbc=TIGHT)
    s.set_h_ext(h)
    return s


def test_one_material_equals_the_single_material_oracle():
    from multimat import MultiOracle
    msh = halves()
    mat = material("Py")
    L = SiteLayer(msh, [["Py"], ["Py"]])
    assert L.n_sites == msh.n_nodes and np.array_equal(L.site_node, np.arange(msh.n_nodes))
    mo = MultiOracle(msh.points, msh.simplices, L, {"Py": mat.coefficients("nmag")})
    h = [0.01, -0.02, 0.03]
    mo.set_h_ext(h)
    m = seeded_m(msh.n_nodes, seed=61, noise=0.5)
    d = mo.rhs(m)
    s = _single_oracle(msh, mat, h)
    ds = s.rhs(m).reshape(-1, 3)
    assert np.abs(d - ds).max() <= 1e-9 * np.abs(ds).max()
    assert np.abs(mo.fields["H_demag"] - s.field("H_demag")).max() <= 1e-9 * np.abs(s.field("H_demag")).max()


def test_materials_on_disjoint_regions_equal_one_material():
    """Two materials with the same constants on regions that do not touch:
    no node has two sites, so the system is the single-material one."""
    from multimat import MultiOracle
    msh = two_boxes()
    L = SiteLayer(msh, [["A"], ["B"]])
    assert L.n_sites == msh.n_nodes
    coeffs = {"A": material("A").coefficients("nmag"), "B": material("B").coefficients("nmag")}
    mo = MultiOracle(msh.points, msh.simplices, L, coeffs)
    m = seeded_m(msh.n_nodes, seed=62, noise=0.4)
    d = mo.rhs(m[L.site_node])
    s = _single_oracle(msh, material("Py"), [0.0, 0.0, 0.0])
    ds = s.rhs(m).reshape(-1, 3)[L.site_node]
    assert np.abs(d - ds).max() <= 1e-9 * np.abs(ds).max()


def test_interface_charges_cancel_for_equal_magnetisation():
    """Halves with equal Ms and a uniform m: the surface charges of the two
    sides cancel on the interface, so rho and H_demag are those of one
    material; with different Ms the interface carries (Ms_A - Ms_B) m.n and
    the total charge stays zero."""
    from multimat import MultiOracle
    msh = halves()
    L = SiteLayer(msh, [["A"], ["B"]])
    m_node = np.tile(np.array([0.8, 0.36, 0.48]), (msh.n_nodes, 1))
    same = MultiOracle(msh.points, msh.simplices, L, {"A": material("A").coefficients("nmag"),
                                                       "B": material("B").coefficients("nmag")})
    one = MultiOracle(msh.points, msh.simplices, SiteLayer(msh, [["P"], ["P"]]),
                      {"P": material("P").coefficients("nmag")})
    same.rhs(m_node[L.site_node])
    one.rhs(m_node)
    scale = np.abs(one.fields["rho"]).max()
    assert np.abs(same.fields["rho"] - one.fields["rho"]).max() <= 1e-12 * scale
    assert np.abs(same.fields["H_demag"] - one.fields["H_demag"]).max() <= 1e-10 * np.abs(one.fields["H_demag"]).max()
    diff = MultiOracle(msh.points, msh.simplices, L, {"A": material("A").coefficients("nmag"),
                                                       "B": material("B", Ms=4.3e5).coefficients("nmag")})
    diff.rhs(m_node[L.site_node])
    rho = diff.fields["rho"]
    assert abs(rho.sum()) <= 1e-12 * np.abs(rho).sum()
    x = msh.points[:, 0]
    changed = np.abs(rho - one.fields["rho"]) > 1e-12 * scale
    assert np.any(changed[x == 6.0])


def test_no_exchange_across_the_interface():
    from multimat import MultiOracle
    msh = halves()
    L = SiteLayer(msh, [["A"], ["B"]])
    mo = MultiOracle(msh.points, msh.simplices, L, {"A": material("A").coefficients("nmag"),
                                                     "B": material("B").coefficients("nmag")})
    m = seeded_m(L.n_sites, seed=63, noise=0.3)
    mo.rhs(m)
    h0 = mo.fields["H_exch"].copy()
    k = int(np.nonzero(msh.points[:, 0] == 6.0)[0][0])
    sa, sb = L.node_site_idx[L.node_site_ptr[k]:L.node_site_ptr[k + 1]]
    m2 = m.copy()
    m2[sa] = [0.0, 0.0, 1.0]                      # turn A's interface spin only
    mo.rhs(m2)
    h1 = mo.fields["H_exch"]
    b_sites = L.sites_of("B")
    assert np.array_equal(h1[b_sites], h0[b_sites])
    assert np.abs(h1[L.sites_of("A")] - h0[L.sites_of("A")]).max() > 0.0


def test_sites_where_each_material_is_defined():
    """The expectations of interface/nmag/test_fefields.py on a two-region
    mesh: a subfield on region A, one on region B and one on both; setting
    one at a node works exactly where its material is defined (interface
    nodes belong to both regions)."""
    msh = halves()
    L = SiteLayer(msh, [["ab", "a"], ["ab", "b"]])
    x = msh.points[:, 0]
    for node in range(msh.n_nodes):
        in_a, in_b = x[node] <= 6.0, x[node] >= 6.0
        assert L.site_node[L.site_index("ab", node)] == node
        for name, defined in (("a", in_a), ("b", in_b)):
            if defined:
                assert L.site_node[L.site_index(name, node)] == node
            else:
                with pytest.raises(KeyError):
                    L.site_index(name, node)


def test_local_coupling_coefficients_host_side():
    """Simulation.set_local_magnetic_coupling's coefficients against the
    reference's formula (main.py:1234-1263): c = coupling / mu0, H_lc of
    material 1 gains c Ms_2 (simulation units) and E_lc the energy density
    0.5 mu0 Ms_1 Ms_2 times c, and the other way round; a pair gives one
    coupling per direction; a second coupling of the same pair, a material
    with itself, or a one-material simulation is refused.  The engine is a
    stand-in that records the calls (no GPU)."""
    from nmag import si, simulation_units
    a = nmag.MagMaterial("A", Ms=SI(6e5, "A/m"), exchange_coupling=SI(1.0e-11, "J/m"))
    b = nmag.MagMaterial("B", Ms=SI(1.0e6, "A/m"), exchange_coupling=SI(1.5e-11, "J/m"))
    c = nmag.MagMaterial("C", Ms=SI(8e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"))

    class Recorder:
        def __init__(self):
            self.calls = []

        def set_local_coupling(self, k1, k2, h, e):
            self.calls.append((k1, k2, h, e))

    sim = nmag.Simulation("lc")
    with pytest.raises(KeyError):   # one material: no sites to couple
        sim.set_local_magnetic_coupling(a, b, SI(-0.5e-6, "N/A^2"))
    sim.layer = object()
    sim.materials = [a, b, c]
    sim.engine = Recorder()
    sim.set_local_magnetic_coupling(a, b, SI(-0.5e-6, "N/A^2"))
    sim.set_local_magnetic_coupling(c, a, (SI(-0.2e-6, "N/A^2"), SI(-0.3e-6, "N/A^2")))
    mu0 = 4e-7 * np.pi
    su_Ms = {m.name: simulation_units.of(m.Ms, compatible_with=SI("A/m")) for m in (a, b, c)}

    def en(m1, m2):
        return simulation_units.of(0.5 * si.mu0 * m1.Ms * m2.Ms, compatible_with=SI("J/m^3"))

    want = [(0, 1, -0.5e-6 / mu0 * su_Ms["B"], -0.5e-6 / mu0 * en(a, b)),
            (1, 0, -0.5e-6 / mu0 * su_Ms["A"], -0.5e-6 / mu0 * en(a, b)),
            (2, 0, -0.2e-6 / mu0 * su_Ms["A"], -0.2e-6 / mu0 * en(c, a)),
            (0, 2, -0.3e-6 / mu0 * su_Ms["C"], -0.3e-6 / mu0 * en(c, a))]
    assert len(sim.engine.calls) == 4
    for got, exp in zip(sim.engine.calls, want):
        assert got[:2] == exp[:2]
        assert np.allclose(got[2:], exp[2:], rtol=1e-12, atol=0.0), (got, exp)
    for m1, m2 in ((b, a), (a, b), (a, a)):
        with pytest.raises(ValueError):
            sim.set_local_magnetic_coupling(m1, m2, SI(-0.1e-6, "N/A^2"))
