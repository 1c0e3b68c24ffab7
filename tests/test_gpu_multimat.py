"""Several magnetic materials on the GPU (nmg_create_materials) against the
oracle's multi-material right-hand side (oracle/multimat.py: every material's
own m on its sites, exchange within a material, charges of all materials on
one potential; interface/nmag/nmag_lam.py:183-470, 587-606, 734-832).

Poisson solves at 1e-12 on the device (the oracle solves directly), so the
fields agree to 1e-9 relative (max norm); the BDF trajectory at rtol = atol =
1e-8 against the oracle's right-hand side integrated by scipy (rtol 1e-11) to
1e-6."""
import numpy as np
import pytest

import nmag
from nmag import SI
from nmag.mesh import Mesh, box_mesh
from nmag.sites import SiteLayer
from conftest import seeded_m

pytestmark = pytest.mark.gpu


def halves():
    """A 12 x 6 x 4 nm box split at x = 6 nm into regions 1 and 2."""
    b = box_mesh(6, 3, 2, 2.0)
    cx = b.points[b.simplices].mean(1)[:, 0]
    return Mesh(b.points, b.simplices, np.where(cx < 6.0, 1, 2))


def two_boxes():
    a = box_mesh(3, 3, 2, 2.0)
    b = box_mesh(3, 3, 2, 2.0, origin=(10.0, 0.0, 0.0))
    pts = np.concatenate([a.points, b.points])
    sim = np.concatenate([a.simplices, b.simplices + a.n_nodes])
    reg = np.concatenate([np.ones(a.n_tets, np.int32), np.full(b.n_tets, 2, np.int32)])
    return Mesh(pts, sim, reg)


def materials():
    py = nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=0.3,
                          llg_gamma_G=SI(2.211e5, "m/A s"))
    co = nmag.MagMaterial("Co", Ms=SI(1.4e6, "A/m"), exchange_coupling=SI(3.0e-11, "J/m"), llg_damping=0.1,
                          llg_gamma_G=SI(2.211e5, "m/A s"),
                          anisotropy=nmag.uniaxial_anisotropy(axis=[0.0, 0.6, 0.8], K1=SI(5e5, "J/m^3")))
    return py, co


def struct(mat):
    from nmag import _lib
    c = mat.coefficients("nmag")
    mt = _lib.Material()
    mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c["Ms"], c["exch_coeff"], c["C1"], c["C2"], c["C3"]
    mt.K1, mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = c["K1"], c["anis_coeff"], c["E_coeff_half"], c["E_coeff_ext"]
    for d in range(3):
        mt.axis[d] = c["axis"][d]
    return mt


def options(B=1, tol=1e-12):
    from nmag import _lib
    op = _lib.Options()
    op.do_demag = 1
    op.nbc_rtol = op.dbc_rtol = tol
    op.nbc_atol = op.dbc_atol = 1e-50
    op.nbc_maxits = op.dbc_maxits = 20000
    op.n_members = B if B > 1 else 0
    return op


def engine(msh, region_mats, mats, B=1):
    from nmag import _lib
    return _lib.Engine.materials(msh.points, msh.simplices, msh.regions, region_mats, [struct(m) for m in mats],
                                 options(B))


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("geometry", ["halves", "two_boxes"])
def test_fields_match_multimaterial_oracle(geometry):
    from multimat import MultiOracle
    msh = halves() if geometry == "halves" else two_boxes()
    py, co = materials()
    eng = engine(msh, [[0], [1]], [py, co])
    L = SiteLayer(msh, [["Py"], ["Co"]])
    node, mat = eng.site_info()
    assert eng.N == L.n_sites
    assert np.array_equal(node, L.site_node) and np.array_equal(mat, L.site_material)
    mo = MultiOracle(msh.points, msh.simplices, L, {"Py": py.coefficients("nmag"), "Co": co.coefficients("nmag")})
    h = np.array([0.02, -0.01, 0.03])
    mo.set_h_ext(h)
    eng.set_h_ext(h)
    m = seeded_m(L.n_sites, base=(0.3, 1.0, -0.2), seed=71, noise=0.4)
    eng.set_m(m)
    f = eng.eval_fields()
    d = mo.rhs(m)
    for key in ("H_exch", "H_anis", "H_total"):
        assert rel(f[key], mo.fields[key]) < 1e-9, (key, rel(f[key], mo.fields[key]))
    # H_demag lives on the mesh nodes in the oracle: every site carries its node's
    assert rel(f["H_demag"], mo.fields["H_demag"][L.site_node]) < 1e-9
    assert rel(f["dmdt"], d) < 1e-9
    assert rel(f["rho"], mo.fields["rho_sites"]) < 1e-9
    assert rel(f["phi"], mo.fields["phi"][L.site_node]) < 1e-9
    # per-material averages and energies: volume sums over each material's sites
    E = eng.energy_density()
    for k, name in enumerate(("Py", "Co")):
        s = L.sites_of(name)
        V = np.asarray(eng.csr()[5])[s]
        a, e = eng.material_averages(k, energies=True)
        assert np.allclose(a, (m[s] * V[:, None]).sum(0) / V.sum(), rtol=1e-12)
        assert np.allclose(e[4], (E["E_total"][s] * V).sum(), rtol=1e-12)
    eng.close()


def test_one_material_over_two_regions_equals_the_single_handle():
    from test_gpu_parity import make_engine
    msh = halves()
    py, _ = materials()
    eng = engine(msh, [[0], [0]], [py])
    single = make_engine(msh, py)
    assert eng.N == msh.n_nodes
    m = seeded_m(msh.n_nodes, seed=72, noise=0.4)
    for e in (eng, single):
        e.set_h_ext([0.01, 0.0, -0.02])
        e.set_m(m)
    f, g = eng.eval_fields(), single.eval_fields()
    assert rel(f["dmdt"], g["dmdt"]) < 1e-12
    eng.close()
    single.close()


def test_rk4_and_bdf_trajectories_match_multimaterial_oracle():
    """Fixed-step RK4 on the device (nmg_rk4_device) against the same scheme
    driven by the oracle's right-hand side (1e-9: the same arithmetic up to
    rounding and the Poisson solves); then the device's BDF (rtol = atol =
    1e-8) against the oracle's right-hand side integrated to 1e-11 by scipy,
    within the metric's 1e-4 (the BDF's own global error in this fast
    transient, with the anisotropic Co half, is ~1e-5)."""
    import torch
    from scipy.integrate import solve_ivp
    from multimat import MultiOracle
    msh = halves()
    py, co = materials()
    eng = engine(msh, [[0], [1]], [py, co])
    L = SiteLayer(msh, [["Py"], ["Co"]])
    mo = MultiOracle(msh.points, msh.simplices, L, {"Py": py.coefficients("nmag"), "Co": co.coefficients("nmag")})
    h = np.array([0.0, 0.05, 0.0])
    mo.set_h_ext(h)
    eng.set_h_ext(h)
    m0 = seeded_m(L.n_sites, base=(1.0, 0.2, 0.1), seed=73, noise=0.2)
    dt, steps = 0.01, 50
    d = torch.tensor(m0.reshape(-1), dtype=torch.float64, device="cuda")
    eng.rk4_device(int(d.data_ptr()), dt, steps)
    m_dev = d.cpu().numpy().reshape(-1, 3)
    y = m0.reshape(-1).copy()
    f = lambda v: mo.rhs(v).reshape(-1)
    for _ in range(steps):
        k1 = f(y); k2 = f(y + 0.5 * dt * k1); k3 = f(y + 0.5 * dt * k2); k4 = f(y + dt * k3)
        y = y + dt / 6.0 * (((k1 + 2.0 * k2) + 2.0 * k3) + k4)
    assert np.abs(m_dev - y.reshape(-1, 3)).max() < 1e-9
    eng.set_m(m0)
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    ref = solve_ivp(lambda t, v: f(v), (0.0, 5.0), m0.reshape(-1), method="DOP853",
                    rtol=1e-11, atol=1e-11, t_eval=[1.0, 2.5, 5.0])
    for k, t in enumerate((1.0, 2.5, 5.0)):
        eng.ts_advance(t)
        diff = np.abs(eng.get_m() - ref.y[:, k].reshape(-1, 3)).max()
        print("several materials, BDF at 1e-8 against the converged solution, t = %.1f ps: %.2e" % (t, diff))
        assert diff < 1e-4, (t, diff)
    assert np.abs(ref.y[:, -1].reshape(-1, 3) - m0).max() > 1e-2   # the state moved
    eng.close()


def test_ensemble_members_equal_single_multimaterial_handles():
    msh = halves()
    py, co = materials()
    ens = engine(msh, [[0], [1]], [py, co], B=2)
    S = ens.N
    ms = np.stack([seeded_m(S, base=(1.0, 0.1 * b, 0.3), seed=80 + b, noise=0.3) for b in range(2)])
    ens.set_h_ext(np.zeros(3))
    ens.set_m(ms)
    f = ens.eval_fields()
    for b in range(2):
        one = engine(msh, [[0], [1]], [py, co])
        one.set_h_ext(np.zeros(3))
        one.set_m(ms[b])
        g = one.eval_fields()
        assert rel(f["dmdt"][b], g["dmdt"]) < 1e-9
        one.close()
    ens.close()


def test_simulation_api_with_two_materials(tmp_path, monkeypatch):
    """nmag.Simulation with two materials on two regions: m per material,
    per-material subfields and averages, advance_time, the .ndt row."""
    monkeypatch.chdir(tmp_path)
    msh = halves()
    py, co = materials()
    sim = nmag.Simulation("two", ksp_tolerances={"NBC.rtol": 1e-10, "DBC.rtol": 1e-10})
    sim.load_mesh(msh, [("left", py), ("right", co)], unit_length=SI(1e-9, "m"))
    L = SiteLayer(msh, [["Py"], ["Co"]])
    assert sim.engine.N == L.n_sites
    sim.set_m([1.0, 0.0, 0.0])
    sim.set_m([0.0, 1.0, 0.0], subfieldname="m_Co")
    assert np.allclose(sim.get_subfield("m_Py"), [1.0, 0.0, 0.0])
    assert np.allclose(sim.get_subfield("m_Co"), [0.0, 1.0, 0.0])
    assert np.allclose(sim.get_subfield_average_siv("m", "Co"), [0.0, 1.0, 0.0])
    assert sim.get_subfield("H_demag").shape == (msh.n_nodes, 3)
    sim.set_H_ext([0.0, 0.0, 1e5], SI(1.0, "A/m"))
    t = sim.advance_time(SI(2e-12, "s"))
    assert abs(t.value - 2e-12) < 1e-24
    mpy, mco = sim.get_subfield("m_Py"), sim.get_subfield("m_Co")
    assert np.abs(np.linalg.norm(mpy, axis=1) - 1).max() < 1e-4 and np.abs(np.linalg.norm(mco, axis=1) - 1).max() < 1e-4
    sim.save_data()
    header = open("two_dat.ndt").readline()
    for col in ("m_Py_0", "m_Co_1", "H_demag_0", "maxangle_m_Py", "maxangle_m_Co"):
        assert col in header
    sim.set_damping(1.0)
    sim.relax()   # the default saves: averages and every field at the stage end
    assert sim.clock.convergence
    from nmag import h5data
    saved = h5data.read(str(tmp_path / "two_dat.h5"))["tables"]
    assert saved["m"]["m_Co"][-1].shape == (len(L.sites_of("Co")), 3)
    assert saved["H_demag"]["H_demag"][-1].shape == (msh.n_nodes, 3)


def test_local_coupling_matches_oracle():
    """Two species on the same nodes (region 1 carries A and B, region 2
    only B) coupled locally (nmag_lam.py:16-62): H_lc of each species from
    the other's m at the shared nodes, in H_total and dm/dt against the
    oracle (1e-9); the energy density's E_lc against the oracle's."""
    from multimat import MultiOracle
    msh = halves()
    a = nmag.MagMaterial("A", Ms=SI(6e5, "A/m"), exchange_coupling=SI(1.0e-11, "J/m"), llg_damping=0.2,
                         llg_gamma_G=SI(2.211e5, "m/A s"))
    b = nmag.MagMaterial("B", Ms=SI(1.0e6, "A/m"), exchange_coupling=SI(1.5e-11, "J/m"), llg_damping=0.2,
                         llg_gamma_G=SI(2.211e5, "m/A s"))
    L = SiteLayer(msh, [["A", "B"], ["B"]])
    coup = {("A", "B"): (-0.3, -0.12), ("B", "A"): (-0.2, -0.08)}
    engs = []
    for couple in (False, True):
        e = engine(msh, [[0, 1], [1]], [a, b])
        if couple:
            for (x, y), (hc, ec) in coup.items():
                e.set_local_coupling("AB".index(x), "AB".index(y), hc, ec)
        engs.append(e)
    mo = MultiOracle(msh.points, msh.simplices, L, {"A": a.coefficients("nmag"), "B": b.coefficients("nmag")})
    for (x, y), (hc, ec) in coup.items():
        mo.set_local_coupling(x, y, hc, ec)
    m = seeded_m(L.n_sites, base=(0.2, 1.0, 0.4), seed=91, noise=0.5)
    h = np.array([0.01, 0.0, -0.02])
    mo.set_h_ext(h)
    for e in engs:
        e.set_h_ext(h)
        e.set_m(m)
    f0, f = engs[0].eval_fields(), engs[1].eval_fields()
    d = mo.rhs(m)
    assert np.abs(mo.fields["H_lc"]).max() > 0.05   # the coupling is felt
    assert rel(f["H_total"], mo.fields["H_total"]) < 1e-9
    assert rel(f["dmdt"], d) < 1e-9
    assert np.abs((f["H_total"] - f0["H_total"]) - mo.fields["H_lc"]).max() < 1e-12
    E0, E1 = engs[0].energy_density()["E_total"], engs[1].energy_density()["E_total"]
    assert np.abs((E1 - E0) - mo.fields["E_lc"]).max() < 1e-12
    for e in engs:
        e.close()


def test_simulation_local_magnetic_coupling(tmp_path, monkeypatch):
    """Simulation.set_local_magnetic_coupling (main.py:1234-1263) on two
    species sharing region 1: the coefficients reach the device (the H_total
    difference from an uncoupled run is the coupling field) and the
    dynamics run."""
    monkeypatch.chdir(tmp_path)
    msh = halves()
    a = nmag.MagMaterial("A", Ms=SI(6e5, "A/m"), exchange_coupling=SI(1.0e-11, "J/m"), llg_damping=0.2)
    b = nmag.MagMaterial("B", Ms=SI(1.0e6, "A/m"), exchange_coupling=SI(1.5e-11, "J/m"), llg_damping=0.2)
    sims = []
    for couple in (False, True):
        sim = nmag.Simulation("lc%d" % couple, ksp_tolerances={"NBC.rtol": 1e-12, "DBC.rtol": 1e-12})
        sim.load_mesh(msh, [("r1", [a, b]), ("r2", b)], unit_length=SI(1e-9, "m"))
        if couple:
            sim.set_local_magnetic_coupling(a, b, SI(-0.5e-6, "N/A^2"))
            with pytest.raises(ValueError):
                sim.set_local_magnetic_coupling(b, a, SI(-0.5e-6, "N/A^2"))
        sim.set_m([1.0, 0.2, 0.0], subfieldname="m_A")
        sim.set_m([-0.3, 1.0, 0.1], subfieldname="m_B")
        sims.append(sim)
    L = SiteLayer(msh, [["A", "B"], ["B"]])
    mA = sims[1].get_subfield("m_A")
    dH = sims[1].get_subfield("H_total_A") - sims[0].get_subfield("H_total_A")
    nodeB = {L.site_node[s]: k for k, s in enumerate(L.sites_of("B"))}
    mB = sims[1].get_subfield("m_B")
    c = (-0.5e-6 / (4e-7 * np.pi)) * 1.0e6   # (coupling / mu0) Ms_B in A/m per unit m_B
    exp = np.array([c * mB[nodeB[L.site_node[s]]] for s in L.sites_of("A")])
    assert np.abs(dH - exp).max() <= 1e-9 * np.abs(exp).max()
    t = sims[1].advance_time(SI(1e-12, "s"))
    assert abs(t.value - 1e-12) < 1e-24
    assert np.abs(np.linalg.norm(sims[1].get_subfield("m_A"), axis=1) - 1).max() < 1e-4
