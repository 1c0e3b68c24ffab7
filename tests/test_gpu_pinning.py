"""Pinning field on the GPU (nmg_set_pinning): the factor pin of dm/dt in
k_heff_llg and of the Jacobian rows in k_jv_psolve / k_pprep, against the
oracle's RHS and BDF trajectory; pinned nodes keep their magnetisation."""
import numpy as np
import pytest

import nmag
from nmag import SI
from conftest import permalloy, seeded_m
from test_gpu_parity import make_engine

pytestmark = pytest.mark.gpu


def test_pinned_rhs_matches_oracle(cube):
    import oracle
    mat = permalloy(0.3)
    c = mat.coefficients("nmag")
    eng = make_engine(cube, mat)
    N = cube.n_nodes
    pin = np.random.default_rng(41).choice([0.0, 1.0, 0.5], size=N)
    m = seeded_m(N, seed=41, noise=0.5)
    eng.set_pinning(pin)
    eng.set_h_ext([0.0, 0.0, 0.03])
    eng.set_m(m)
    f = eng.eval_fields()
    om = oracle.OracleMesh(cube.points, cube.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    s.set_pinning(pin)
    s.set_h_ext([0.0, 0.0, 0.03])
    d = s.rhs(m).reshape(-1, 3)
    assert np.abs(f["dmdt"] - d).max() <= 1e-9 * np.abs(d).max()
    assert np.all(f["dmdt"][pin == 0.0] == 0.0)
    # without the field the free nodes' dm/dt is unchanged (the Poisson solves
    # start from the last solution: equal to their tolerance)
    eng.set_pinning(None)
    g = eng.eval_fields()["dmdt"]
    assert np.abs(g[pin == 1.0] - f["dmdt"][pin == 1.0]).max() <= 1e-9 * np.abs(g).max()
    assert np.abs(g[pin == 0.0]).max() > 0.0


def test_pinned_trajectory_matches_oracle(small_box):
    import oracle
    mat = permalloy(0.5)
    c = mat.coefficients("nmag")
    eng = make_engine(small_box, mat)
    om = oracle.OracleMesh(small_box.points, small_box.simplices)
    s = oracle.OracleSim(om, c, nbc=(1e-12, 1e-50, 20000), dbc=(1e-12, 1e-50, 20000))
    N = small_box.n_nodes
    pin = (small_box.points[:, 0] > 3.0).astype(np.float64)   # the x <= 3 nm end held fixed
    m0 = seeded_m(N, base=(1.0, 0.4, 0.3), seed=42, noise=0.5)
    for e in (eng, s):
        e.set_pinning(pin)
        e.set_h_ext([0.0, 0.0, 0.05])
    eng.set_m(m0)
    eng.ts_init(0.0, 1e-8, 1e-8, 2, 300)
    s.ts_init(m0, rtol=1e-8, atol=1e-8)
    for t in (2.0, 8.0):
        _, st = eng.ts_advance(t)
        _, mo = s.ts_advance(t)
        mg = eng.get_m()
        assert np.abs(mg - mo).max() < 1e-6, (t, st, s.ts_stats())
        assert np.abs(mg[pin == 0.0] - m0[pin == 0.0]).max() < 1e-14
        assert np.abs(mg[pin == 1.0] - m0[pin == 1.0]).max() > 1e-3   # the free part moved


def test_simulation_set_pinning():
    from nmag import mesh
    sim = nmag.Simulation()
    sim.load_mesh(mesh.box_mesh(5, 2, 2, 2.0), [("bar", permalloy(0.5))], unit_length=SI(1e-9, "m"))
    sim.set_m([1.0, 0.5, 0.2])
    sim.set_H_ext([0, 0, 5e5], unit=SI("A/m"))
    sim.set_pinning(lambda p: 0.0 if p[0] < 2.5e-9 else 1.0)
    pin = sim.get_subfield("pin")
    assert set(np.unique(pin)) == {0.0, 1.0}
    m0 = sim.engine.get_m().copy()
    sim.advance_time(SI(5e-12, "s"))
    m1 = sim.engine.get_m()
    assert np.abs(m1[pin == 0.0] - m0[pin == 0.0]).max() < 1e-14
    assert np.abs(m1[pin == 1.0] - m0[pin == 1.0]).max() > 1e-3
