"""Spin-transfer torque on the GPU (nmg_set_stt / nmg_set_current_density,
k_stt_dmdc + the C4/C5 terms of k_heff_llg) against the oracle: dm/dt of one
evaluation, the exact (J . grad) m of a linear field, a BDF trajectory, the
ensemble form and the Simulation API."""
import numpy as np
import pytest

import nmag
from nmag import SI
from conftest import seeded_m
from test_gpu_parity import make_engine
from test_stt import stt_material

pytestmark = pytest.mark.gpu


def stt_engine(msh, mat, **kw):
    c = mat.coefficients("nmag")
    eng = make_engine(msh, mat, **kw)
    eng.set_stt(c["C4"], c["C5"])
    return eng, c


def test_stt_rhs_matches_oracle(cube):
    import oracle
    mat = stt_material(alpha=0.1)
    eng, c = stt_engine(cube, mat)
    rng = np.random.default_rng(21)
    J = 3e-2 * rng.standard_normal((cube.n_nodes, 3))   # ~3e13 A/m^2: the torque is ~20% of dm/dt
    m = seeded_m(cube.n_nodes, seed=21, noise=0.6)
    eng.set_current_density(J)
    eng.set_h_ext([0.0, 0.0, 0.02])
    eng.set_m(m)
    f = eng.eval_fields()
    om = oracle.OracleMesh(cube.points, cube.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    s.set_stt(c["C4"], c["C5"], J)
    s.set_h_ext([0.0, 0.0, 0.02])
    d = s.rhs(m).reshape(-1, 3)
    assert np.abs(f["dmdt"] - d).max() <= 1e-9 * np.abs(d).max()
    # the spin-transfer part alone: J = 0 on a second engine
    eng0 = make_engine(cube, mat)
    eng0.set_h_ext([0.0, 0.0, 0.02])
    eng0.set_m(m)
    d0 = eng0.eval_fields()["dmdt"]
    u = s.field("dm_dcurrent")
    mxu = np.cross(m, u)
    part = c["C4"] * np.cross(m, mxu) + c["C5"] * mxu
    assert np.abs(part).max() > 0.1 * np.abs(d0).max()   # the torque matters in this test
    assert np.abs((f["dmdt"] - d0) - part).max() <= 1e-9 * np.abs(part).max()


def test_stt_linear_field_is_exact(small_box):
    mat = stt_material()
    eng, c = stt_engine(small_box, mat, do_demag=False)
    mat0 = nmag.MagMaterial("Py", Ms=SI(8e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=0.02)
    eng0 = make_engine(small_box, mat0, do_demag=False)
    x = small_box.points
    grad = np.array([[0.3, -0.1, 0.2], [0.05, 0.4, -0.3], [-0.2, 0.1, 0.15]])
    m = np.array([1.0, 0.5, -0.4])[None, :] + x @ grad.T
    J = np.array([2e-3, -1e-3, 5e-4])
    eng.set_current_density(J)
    for e in (eng, eng0):
        e.set_h_ext(np.zeros(3))
        e.set_m(m)
    u = (grad @ J)[None, :]
    mxu = np.cross(m, u)
    part = c["C4"] * np.cross(m, mxu) + c["C5"] * mxu
    diff = eng.eval_fields()["dmdt"] - eng0.eval_fields()["dmdt"]
    assert np.abs(diff - part).max() <= 1e-12 * np.abs(part).max()
    # zero current: no torque; switching the coefficients off likewise
    eng.set_current_density(None)
    assert np.abs(eng.eval_fields()["dmdt"] - eng0.eval_fields()["dmdt"]).max() == 0.0
    eng.set_current_density(J)
    eng.set_stt(0.0, 0.0)
    assert np.abs(eng.eval_fields()["dmdt"] - eng0.eval_fields()["dmdt"]).max() == 0.0


def test_stt_trajectory_matches_oracle(small_box):
    import oracle
    mat = stt_material(alpha=0.3, P=1.0, xi=0.1)
    eng, c = stt_engine(small_box, mat)
    om = oracle.OracleMesh(small_box.points, small_box.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    J = np.array([5e-3, 1e-3, 0.0])   # 5e12 A/m^2
    s.set_stt(c["C4"], c["C5"], J)
    eng.set_current_density(J)
    m0 = seeded_m(small_box.n_nodes, base=(1.0, 0.3, 0.2), seed=22, noise=0.5)
    eng.set_h_ext(np.zeros(3))
    s.set_h_ext(np.zeros(3))
    eng.set_m(m0)
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    s.ts_init(m0, rtol=1e-8, atol=1e-8)
    for t in (2.0, 6.0):
        _, st = eng.ts_advance(t)
        _, mo = s.ts_advance(t)
        assert np.abs(eng.get_m() - mo).max() < 1e-6, (t, st, s.ts_stats())


def test_stt_ensemble_matches_single(cube):
    from test_gpu_ensemble import make_ensemble, _members
    mat = stt_material(alpha=0.1)
    c = mat.coefficients("nmag")
    B = 2
    ens, single = make_ensemble(cube, mat, B)
    ens.set_stt(c["C4"], c["C5"])
    single.set_stt(c["C4"], c["C5"])
    ms, hs = _members(cube.n_nodes, B, seed0=500)
    Js = np.stack([np.broadcast_to([3e-3 * (b + 1), -1e-3, 0.0], (cube.n_nodes, 3)) for b in range(B)])
    ens.set_m(ms)
    ens.set_h_ext(hs)
    ens.set_current_density(Js)
    f = ens.eval_fields()
    for b in range(B):
        single.set_m(ms[b])
        single.set_h_ext(hs[b])
        single.set_current_density(Js[b])
        g = single.eval_fields()
        assert np.abs(f["dmdt"][b] - g["dmdt"]).max() <= 1e-9 * np.abs(g["dmdt"]).max(), b


def test_simulation_current_density():
    from nmag import mesh
    sim = nmag.Simulation()
    sim.load_mesh(mesh.box_mesh(6, 2, 2, 2.0), [("bar", stt_material(alpha=0.1))], unit_length=SI(1e-9, "m"))
    sim.set_m(lambda p: [1.0, float(np.sin(p[0] * 1e8)), 0.2])
    sim.set_current_density([1e12, 0, 0], unit=SI("A/m^2"))
    j = sim.get_subfield("current_density")
    assert np.allclose(j, [[1e12, 0, 0]], rtol=1e-12)
    d1 = sim.engine.eval_fields()["dmdt"]
    sim.set_current_density([0, 0, 0], unit=SI("A/m^2"))
    d0 = sim.engine.eval_fields()["dmdt"]
    assert np.abs(d1 - d0).max() > 1e-3 * np.abs(d0).max()
    sim.set_current_density([SI(1e12, "A/m^2"), SI(0, "A/m^2"), SI(0, "A/m^2")])
    assert np.abs(sim.engine.eval_fields()["dmdt"] - d1).max() <= 1e-12 * np.abs(d1).max()
    sim.advance_time(SI(2e-12, "s"))


def test_adjoint_refuses_stt(small_box):
    torch = pytest.importorskip("torch")
    from nmag import NmagGpuError
    eng, _ = stt_engine(small_box, stt_material())
    eng.set_current_density([1e-3, 0.0, 0.0])
    n3 = 3 * small_box.n_nodes
    m0 = torch.tensor(seeded_m(small_box.n_nodes, seed=23).reshape(-1), dtype=torch.float64, device="cuda")
    mT = torch.zeros(n3, dtype=torch.float64, device="cuda")
    with pytest.raises(NmagGpuError):
        eng.rk4_forward(m0.data_ptr(), 0.1, 2, 1, 0, 0, 1, mT.data_ptr(), 0)
