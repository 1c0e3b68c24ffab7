"""Polynomial anisotropy on the GPU (nmg_set_anisotropy_poly): the field and
energy density of k_anis_poly / k_energy against the tables evaluated on the
host and against the oracle, a trajectory against the oracle's BDF, the
ensemble form, and the second-order polynomial against the closed-form K1
path."""
import numpy as np
import pytest

import nmag
from nmag import SI
from nmag.anisotropy import polynomial_tables
from conftest import seeded_m
from test_anisotropy import eval_tables
from test_gpu_parity import make_engine

pytestmark = pytest.mark.gpu


def cubic_material(alpha=0.5):
    return nmag.MagMaterial("Fe", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(2.211e5, "m/A s"),
                            anisotropy=nmag.cubic_anisotropy([1, 0.2, 0], [0, 1, 0.3], K1=SI(-2.5e5, "J/m^3"),
                                                             K2=SI(8e4, "J/m^3"), K3=SI(3e4, "J/m^3")))


def uniaxial4_material(alpha=0.5):
    return nmag.MagMaterial("Co", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_gamma_G=SI(2.211e5, "m/A s"),
                            anisotropy=nmag.uniaxial_anisotropy([0.2, 0.3, 1.0], K1=SI(3e5, "J/m^3"),
                                                                K2=SI(1e5, "J/m^3")))


@pytest.mark.parametrize("make_mat", [cubic_material, uniaxial4_material])
def test_poly_field_and_energy_match_tables_and_oracle(cube, make_mat):
    import oracle
    mat = make_mat()
    c = mat.coefficients("nmag")
    eng = make_engine(cube, mat)
    m = seeded_m(cube.n_nodes, seed=11, noise=1.0)
    eng.set_h_ext([0.01, -0.02, 0.03])
    eng.set_m(m)
    f = eng.eval_fields()
    E, H = eval_tables(c["anis_poly"], m)
    # the order-8 cubic table sums ~90 terms whose coefficients add up to
    # ~700 max|H|: rounding differences of the summation order reach ~1e-13
    scale = np.abs(H).max()
    assert np.abs(f["H_anis"] - H).max() <= 1e-12 * scale
    assert np.abs(f["H_total"] - (f["H_exch"] + f["H_demag"] + f["H_anis"] + np.array([0.01, -0.02, 0.03]))).max() \
        <= 1e-13 * np.abs(f["H_total"]).max()
    Ed = eng.energy_density()
    assert np.abs(Ed["E_anis"] - E).max() <= 1e-12 * np.abs(E).max()
    # the oracle evaluates the same tables as the reference's generated code
    om = oracle.OracleMesh(cube.points, cube.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    s.set_h_ext([0.01, -0.02, 0.03])
    d = s.rhs(m).reshape(-1, 3)
    assert np.abs(f["H_anis"] - s.field("H_anis")).max() <= 1e-12 * scale
    assert np.abs(f["dmdt"] - d).max() <= 1e-9 * np.abs(d).max()


def test_second_order_polynomial_matches_closed_form(small_box):
    """The uniaxial K1 anisotropy as a polynomial (material K1 = 0) gives the
    closed-form engine's fields and trajectory."""
    from nmag import _lib
    ax = [0.3, 0.4, 0.866]
    mat = nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=0.3,
                           llg_gamma_G=SI(2.211e5, "m/A s"),
                           anisotropy=nmag.uniaxial_anisotropy(ax, K1=SI(4e5, "J/m^3")))
    closed = make_engine(small_box, mat)
    c = mat.coefficients("nmag")
    poly = make_engine(small_box, mat)
    mt = _lib.Material()
    mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c["Ms"], c["exch_coeff"], c["C1"], c["C2"], c["C3"]
    mt.K1, mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = 0.0, 0.0, c["E_coeff_half"], c["E_coeff_ext"]
    poly.set_material(mt)
    T = polynomial_tables(mat.anisotropy.function, 2, 1.0 / (mat.su_mu0 * mat.su_Ms), quirks=None)
    poly.set_anisotropy_poly(*T)
    m = seeded_m(small_box.n_nodes, seed=12, noise=0.8)
    for e in (closed, poly):
        e.set_h_ext([0.0, 0.05, 0.0])
        e.set_m(m)
    fc, fp = closed.eval_fields(), poly.eval_fields()
    assert np.abs(fc["H_anis"] - fp["H_anis"]).max() <= 1e-13 * np.abs(fc["H_anis"]).max()
    assert np.abs(fc["dmdt"] - fp["dmdt"]).max() <= 1e-13 * np.abs(fc["dmdt"]).max()
    assert np.abs(closed.energy_density()["E_anis"] - poly.energy_density()["E_anis"]).max() <= 1e-13
    for e in (closed, poly):
        e.ts_init(0.0, 1e-8, 1e-8, 2, 300)
        e.ts_advance(8.0)
    # RHS equal to ~1e-15: the same steps unless an error test sits on its
    # threshold, when the two paths part by about the local tolerance
    assert np.abs(closed.get_m() - poly.get_m()).max() < 1e-6
    # removing the polynomial leaves no anisotropy
    poly.set_anisotropy_poly()
    poly.set_m(m)
    assert np.abs(poly.eval_fields()["H_anis"]).max() == 0.0


def test_poly_trajectory_matches_oracle(small_box):
    import oracle
    mat = cubic_material(alpha=0.5)
    c = mat.coefficients("nmag")
    eng = make_engine(small_box, mat)
    om = oracle.OracleMesh(small_box.points, small_box.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    m0 = seeded_m(small_box.n_nodes, base=(1.0, 0.2, 0.5), seed=13, noise=0.3)
    eng.set_h_ext(np.zeros(3))
    s.set_h_ext(np.zeros(3))
    eng.set_m(m0)
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    s.ts_init(m0, rtol=1e-8, atol=1e-8)
    for t in (2.0, 6.0):
        _, st = eng.ts_advance(t)
        _, mo = s.ts_advance(t)
        assert np.abs(eng.get_m() - mo).max() < 1e-6, (t, st, s.ts_stats())


def test_poly_ensemble_matches_single(cube):
    from test_gpu_ensemble import make_ensemble, _members
    mat = cubic_material()
    B = 3
    ens, single = make_ensemble(cube, mat, B)
    ms, hs = _members(cube.n_nodes, B, seed0=400)
    ens.set_m(ms)
    ens.set_h_ext(hs)
    f = ens.eval_fields()
    E = ens.energy_density()["E_anis"]
    for b in range(B):
        single.set_m(ms[b])
        single.set_h_ext(hs[b])
        g = single.eval_fields()
        for k in ("H_anis", "H_total", "dmdt"):
            assert np.abs(f[k][b] - g[k]).max() <= 1e-9 * np.abs(g[k]).max(), (b, k)
        assert np.abs(E[b] - single.energy_density()["E_anis"]).max() <= 1e-12 * np.abs(E[b]).max()


def test_adjoint_refuses_polynomial_anisotropy(small_box):
    torch = pytest.importorskip("torch")
    from nmag import NmagGpuError
    eng = make_engine(small_box, cubic_material())
    n3 = 3 * small_box.n_nodes
    m0 = torch.tensor(seeded_m(small_box.n_nodes, seed=14).reshape(-1), dtype=torch.float64, device="cuda")
    mT = torch.zeros(n3, dtype=torch.float64, device="cuda")
    with pytest.raises(NmagGpuError):
        eng.rk4_forward(m0.data_ptr(), 0.1, 2, 1, 0, 0, 1, mT.data_ptr(), 0)


def test_simulation_relaxes_to_cubic_easy_axis():
    """A single-domain cube (no demag) relaxes from near [1,1,0.3] to the
    nearest easy axis of K1 < 0 cubic anisotropy, a <111> direction."""
    from nmag import mesh
    mat = nmag.MagMaterial("Fe", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=1.0,
                           anisotropy=nmag.cubic_anisotropy([1, 0, 0], [0, 1, 0], K1=SI(-4e5, "J/m^3")))
    sim = nmag.Simulation(do_demag=False)
    sim.load_mesh(mesh.box_mesh(3, 3, 3, 2.0, 2.0, 2.0), [("cube", mat)], unit_length=SI(1e-9, "m"))
    sim.set_m([1.0, 0.8, 0.3])
    sim.advance_time(SI(2e-10, "s"))
    m = sim.engine.get_m().mean(axis=0)
    m /= np.linalg.norm(m)
    assert np.abs(m - np.ones(3) / np.sqrt(3)).max() < 1e-3, m
