"""GPU parity: the sm_103a library (through its C-ABI) against the CPU oracle.

Integer work (CSR pattern, reference-shaped operator patterns, boundary
indices, surface triangles) must be bit-exact.  The assembled P1 values are
also bit-exact: both sides evaluate the same operation order without FMA
contraction.  Floating-point results that pass through CUDA's log/acos or
FMA-contracted kernels are compared with stated relative tolerances:
  BEM matrix entries: 1e-12 of the largest entry
  RHS fields with tight Poisson solves (rtol 1e-12): 1e-9 relative (max-norm)
  m(t) from the BDF integrator vs the oracle's: 1e-6 absolute (rtol = atol = 1e-8)
"""
import math

import numpy as np
import pytest

import oracle
from conftest import permalloy, seeded_m

pytestmark = pytest.mark.gpu


def make_engine(msh, mat, do_demag=True, tol=1e-12, bem_precision=0, jv_precision=0):
    from nmag import _lib
    c = mat.coefficients("nmag")
    mt = _lib.Material()
    mt.Ms, mt.exch_coeff, mt.C1, mt.C2, mt.C3 = c["Ms"], c["exch_coeff"], c["C1"], c["C2"], c["C3"]
    mt.K1, mt.anis_coeff, mt.E_coeff_half, mt.E_coeff_ext = c["K1"], c["anis_coeff"], c["E_coeff_half"], c["E_coeff_ext"]
    for d in range(3):
        mt.axis[d] = c["axis"][d]
    op = _lib.Options()
    op.do_demag = int(do_demag)
    op.nbc_rtol = op.dbc_rtol = tol
    op.nbc_atol = op.dbc_atol = 1e-50
    op.nbc_maxits = op.dbc_maxits = 20000
    op.bem_precision = bem_precision
    op.jv_precision = jv_precision
    eng = _lib.Engine(msh.points, msh.simplices, mt, op)
    if c.get("anis_poly") is not None:
        eng.set_anisotropy_poly(*c["anis_poly"])
    return eng


@pytest.fixture(scope="module")
def cube_pair(cube):
    mat = permalloy(0.5)
    eng = make_engine(cube, mat)
    om = oracle.OracleMesh(cube.points, cube.simplices)
    return eng, om, mat


def rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_csr_and_values_bit_exact(cube_pair):
    eng, om, _ = cube_pair
    rp, ci, K, G, D, V = eng.csr()
    assert eng.nnz == om.nnz == 17191
    assert np.array_equal(rp, om.row_ptr)
    assert np.array_equal(ci, om.col_idx)
    assert np.array_equal(K, om.K)
    assert np.array_equal(G, om.G)
    assert np.array_equal(D, om.D)
    assert np.array_equal(V, om.vol)


@pytest.mark.parametrize("which", range(6))
def test_reference_operator_patterns_bit_exact(cube_pair, which):
    eng, om, mat = cube_pair
    coeff = [-24.0583053511, 0.86, 1.0, 1.0, 1.0, 1.0][which]
    a = eng.export_operator(which, coeff)
    b = om.export_operator(which, coeff)
    assert a[3] == b[3]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2])


def test_boundary_and_triangles_bit_exact(cube_pair):
    eng, om, _ = cube_pair
    nob, tri, nrm, sa = eng.boundary()
    assert eng.nb == om.nb == 602 and eng.nouter == 1200
    assert np.array_equal(nob, om.node_of_b)
    assert eng.ntri == om.ntri
    assert np.array_equal(tri, om.tri)
    assert np.array_equal(nrm, om.tri_normal)
    assert np.allclose(sa, om.solid_angle, rtol=1e-14, atol=0)


def test_bem_matrix_matches(cube_pair):
    eng, om, _ = cube_pair
    B = eng.bem()
    assert np.abs(B - om.bem).max() <= 1e-12 * np.abs(om.bem).max()
    assert np.abs(B.sum(1) + 1.0).max() < 1e-9


@pytest.mark.parametrize("name", ["box", "cube", "plate"])
def test_bem_matrix_matches_reference_stub(name):
    """The device fill against BEM matrices filled by the reference's own
    Lindholm stub (src/bem3d_stubs.c:413-610 driven as bem3d.ml:938-1047;
    tests/golden/ref_bem.npz, made by tests/golden/make_ref_bem.py): sampled
    rows within 1e-12 of the largest entry (CUDA's log/acos against the host
    libm's), row and column sums of the whole matrix likewise."""
    import os
    from nmag import mesh
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_bem.npz"))
    a = g[name + "_args"]
    msh = mesh.box_mesh(int(a[0]), int(a[1]), int(a[2]), *a[3:])
    eng = make_engine(msh, permalloy(0.5))
    B = eng.bem()
    scale = np.abs(g[name + "_bem"]).max()
    assert np.abs(B[g[name + "_rows"]] - g[name + "_bem"]).max() <= 1e-12 * scale
    assert np.abs(B.sum(axis=1) - g[name + "_rowsum"]).max() <= 1e-11 * scale
    assert np.abs(B.sum(axis=0) - g[name + "_colsum"]).max() <= 1e-11 * scale


def test_rhs_fields_match_oracle(cube_pair):
    eng, om, mat = cube_pair
    s = oracle.OracleSim(om, mat.coefficients("nmag"), nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    m = seeded_m(om.n_nodes, seed=0)
    hext = np.tile([0.01, -0.02, 0.03], (om.n_nodes, 1))
    s.set_h_ext(hext)
    eng.set_h_ext(hext)
    eng.set_m(m)
    f = eng.eval_fields()
    d = s.rhs(m)
    assert rel_err(f["H_exch"], s.field("H_exch")) < 1e-12
    assert rel_err(f["H_demag"], s.field("H_demag")) < 1e-9
    assert rel_err(f["H_total"], s.field("H_total")) < 1e-9
    assert rel_err(f["dmdt"], d.reshape(-1, 3)) < 1e-9
    assert rel_err(f["phi"], s.scalar_field("phi")) < 1e-9
    E = eng.energy_density()
    Eo = s.energy_density(m)
    assert rel_err(E["E_total"], Eo[4]) < 1e-9
    avg = eng.averages()
    assert np.allclose(avg, (m * om.vol[:, None]).sum(0) / om.vol.sum(), rtol=1e-13)


def test_uniform_cube_demag_factor_gpu(cube_pair):
    eng, om, _ = cube_pair
    eng.set_h_ext(np.zeros(3))
    eng.set_m(np.tile([0.0, 0.0, 1.0], (om.n_nodes, 1)))
    f = eng.eval_fields()
    avg = (f["H_demag"] * om.vol[:, None]).sum(0) / om.vol.sum() / 0.86
    assert abs(avg[2] + 1 / 3) < 0.01
    assert np.abs(f["H_exch"]).max() < 1e-12


def test_single_spin_integration_matches_analytic(small_box):
    from test_oracle_kat import analytic_spin
    mat = permalloy(0.1)
    eng = make_engine(small_box, mat, do_demag=False)
    c = mat.coefficients("nmag")
    H = 0.5
    eng.set_h_ext([0.0, 0.0, H])
    m0 = np.array([math.sin(1.0), 0.0, math.cos(1.0)])
    eng.set_m(np.tile(m0, (small_box.n_nodes, 1)))
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    for t in (5.0, 20.0, 40.0):
        tr, st = eng.ts_advance(t)
        ref = analytic_spin(t, m0, c["C1"], c["C2"], H)
        assert tr == pytest.approx(t, abs=1e-12)
        assert np.abs(eng.get_m() - ref[None]).max() < 2e-5


def test_bdf_trajectory_matches_oracle(cube_pair):
    eng, om, mat = cube_pair
    s = oracle.OracleSim(om, mat.coefficients("nmag"), nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    m0 = seeded_m(om.n_nodes, seed=0)
    eng.set_h_ext(np.zeros(3))
    s.set_h_ext(np.zeros(3))
    eng.set_m(m0)
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    s.ts_init(m0, rtol=1e-8, atol=1e-8)
    for t in (1.0, 5.0, 10.0):
        _, st = eng.ts_advance(t)
        _, mo = s.ts_advance(t)
        mg = eng.get_m()
        assert np.abs(mg - mo).max() < 1e-6, (t, np.abs(mg - mo).max(), st, s.ts_stats())
    # same algorithm: the step counts agree closely
    so = s.ts_stats()
    assert abs(st["nst"] - so["nst"]) <= max(3, 0.05 * so["nst"])


def test_fp32_bem_precision_form_error(cube_pair, cube):
    _, om, mat = cube_pair
    e32 = make_engine(cube, mat, bem_precision=1)
    e64 = cube_pair[0]
    m = seeded_m(om.n_nodes, seed=7, noise=1.0)
    for e in (e32, e64):
        e.set_h_ext(np.zeros(3))
        e.set_m(m)
    f32, f64 = e32.eval_fields(), e64.eval_fields()
    assert rel_err(f32["H_demag"], f64["H_demag"]) < 1e-5
    assert rel_err(f32["H_total"], f64["H_total"]) < 1e-5


def test_simulation_api_advance_and_relax(small_box, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)   # relax saves averages and fields at the stage end
    import nmag
    from nmag import SI
    mat = nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=1.0)
    sim = nmag.Simulation("api_test")
    sim.load_mesh(small_box, [("box", mat)], unit_length=SI(1e-9, "m"))
    sim.set_m([1.0, 0.3, 0.1])
    sim.set_H_ext([0.0, 0.0, 0.5e6], SI(1.0, "A/m"))
    t = sim.advance_time(SI(5e-12, "s"))
    assert abs(t.value - 5e-12) < 1e-24
    m = sim.get_subfield("m")
    assert np.abs(np.linalg.norm(m, axis=1) - 1).max() < 1e-4
    sim.relax()
    assert sim.max_dm_dt < sim.stopping_dm_dt
    assert (tmp_path / "api_test_dat.ndt").exists()
    avg = sim.get_subfield_average_siv("m")
    assert avg[2] > 0.99


def test_simulation_probe_sites_volumes_timers(small_box, tmp_path):
    """probe_subfield(_siv), get_subfield_sites/positions, material_volume,
    get_timers, save_mesh and do_next_stage (main.py:1228,1570-1700,1904,
    2055-2103,2189,2733)."""
    import nmag
    from nmag import SI
    mat = permalloy(0.5)
    sim = nmag.Simulation("probe")
    sim.load_mesh(small_box, [("box", mat)], unit_length=SI(1e-9, "m"))
    sim.set_m(lambda p: [1.0, 0.2 + 1e8 * p[0], 0.1])     # normalised by set_m
    sim.set_H_ext([0.0, 0.0, 1e5], SI(1.0, "A/m"))
    m = sim.get_subfield("m")
    x = sim.get_subfield_positions("m")                   # metres, site order
    assert np.allclose(x, small_box.points * 1e-9)
    assert np.array_equal(sim.get_subfield_sites("m_Py")[:, 0], np.arange(small_box.n_nodes))
    # at a node the probe returns the node's value; between nodes the P1 interpolant
    k = 5
    assert np.allclose(sim.probe_subfield_siv("m_Py", list(x[k])), m[k], atol=1e-14)
    tet = small_box.simplices[3]
    c = x[tet].mean(0)
    assert np.allclose(sim.probe_subfield_siv("m_Py", list(c)), m[tet].mean(0), atol=1e-14)
    h = sim.get_subfield("H_demag")
    got = sim.probe_subfield("H_demag", [SI(v, "m") for v in c])
    assert np.allclose([g.value for g in got], h[tet].mean(0), rtol=1e-9)
    assert sim.probe_subfield_siv("m", [1.0, 1.0, 1.0]) is None
    assert np.allclose(sim.probe_H_demag_siv(list(c / 1e-9), pos_unit=SI(1e-9, "m")), h[tet].mean(0), rtol=1e-9)
    with pytest.raises(NotImplementedError):
        sim.probe_H_demag_siv([1.0, 1.0, 1.0])
    lo, hi = small_box.points.min(0), small_box.points.max(0)
    assert abs(sim.material_volume("Py") - np.prod(hi - lo)) < 1e-9
    assert sim.material_volume(None) == sim.material_volume("Py")
    sim.advance_time(SI(2e-12, "s"))
    (name, _, secs), = sim.get_timers()
    assert name == "advance_time" and secs > 0.0
    sim.save_mesh(str(tmp_path / "m.nmesh"))
    back = nmag.mesh.load(str(tmp_path / "m.nmesh"))
    assert np.allclose(back.points, small_box.points) and np.array_equal(back.simplices, small_box.simplices)
    sim.do_next_stage()
    assert sim.clock.stage == 2 and sim.clock.stage_step == 0 and sim.clock.stage_time_su == 0.0


def test_max_dm_step_tracks_previous_m(small_box):
    """nmg_max_dm_step: distance to m at the previous call or set_m, on the
    device; equal to the host computation on the same arrays."""
    eng = make_engine(small_box, permalloy(0.5), do_demag=False)
    n = small_box.n_nodes
    m0 = seeded_m(n, seed=5, noise=0.3)
    eng.set_m(m0)
    assert eng.max_dm_step() == 0.0                      # first call: nothing to compare with
    eng.set_h_ext(np.zeros(3))
    eng.ts_init(0.0, 1e-6, 1e-6, 2, 300)
    eng.ts_advance(0.5)
    m1 = eng.get_m()
    d = eng.max_dm_step()
    assert d == pytest.approx(np.sqrt(((m1 - m0) ** 2).sum(1)).max(), rel=1e-15)
    assert d > 0.0
    assert eng.max_dm_step() == 0.0                      # nothing moved since the last call
    m2 = seeded_m(n, seed=6, noise=0.3)
    eng.set_m(m2)                                        # set_m becomes the reference
    assert eng.max_dm_step() == 0.0


def test_vacuum_region_simulates_the_magnetic_part():
    """A mesh with vacuum (region 0) simplices: the Simulation runs on its
    magnetic part, whose per-site arrays are those of the magnetic nodes."""
    import nmag
    from nmag import SI, mesh
    from test_host import _shelled_box
    shelled = _shelled_box()
    part, node_map = mesh.magnetic_part(shelled)
    mat = permalloy(0.5)
    tight = {"NBC.rtol": 1e-12, "DBC.rtol": 1e-12}
    sims = []
    for msh in (shelled, part):
        s = nmag.Simulation("vac", ksp_tolerances=tight)
        s.load_mesh(msh, [("a", mat)], unit_length=SI(1e-9, "m"))
        sims.append(s)
    assert sims[0].engine.N == part.n_nodes
    np.testing.assert_array_equal(sims[0].node_map, node_map)
    m = seeded_m(part.n_nodes, seed=3, noise=0.3)
    H = []
    for s in sims:
        s.set_m(m)
        H.append(s.engine.eval_fields()["H_total"])
    assert np.array_equal(H[0], H[1])
