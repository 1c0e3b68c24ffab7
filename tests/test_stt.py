"""Spin-transfer torque (Zhang-Li terms of nmag_lam.py:417-424 with
dm_dcurrent of :872-903): the material coefficients of main.py:440-451 and
the oracle's dm_dcurrent, which for a field linear in space is (J . grad) m
exactly at every node (the lumped P1 gradient of a linear field is exact).
CPU only."""
import numpy as np
import pytest

import nmag
from nmag import SI


def stt_material(alpha=0.02, P=0.7, xi=0.05):
    return nmag.MagMaterial("Py", Ms=SI(8e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=alpha,
                            llg_polarisation=P, llg_xi=xi)


def test_stt_coefficients():
    a, P, xi, Ms = 0.02, 0.7, 0.05, 8e5
    c = stt_material(a, P, xi).coefficients(None)
    # b = P muB / (e Ms) in m^3/C, times the Gilbert-to-LL factor; simulation
    # units: m/s per A/m^2 -> (1e-9/1e-12) / (1e-3/1e-18) = 1e-12
    b = P * 9.2740094980e-24 / (1.6021765314e-19 * Ms * (1 + xi * xi)) / (1 + a * a) / 1e-12
    assert c["C4"] == pytest.approx(-b * (1 + a * xi), rel=1e-12)
    assert c["C5"] == pytest.approx(-b * (xi - a), rel=1e-12)
    q = stt_material(a, P, xi).coefficients("nmag")
    assert q["C4"] == float("%g" % q["C4"]) and q["C5"] == float("%g" % q["C5"])
    plain = nmag.MagMaterial("Py").coefficients()
    assert plain["C4"] == 0.0 and plain["C5"] == 0.0
    assert nmag.MagMaterial("Py").su_llg_stt_prefactor == 0.0 and stt_material().su_llg_stt_prefactor == 1.0


def test_particle_batches_refuse_stt():
    from nmag import batch
    with pytest.raises(NotImplementedError):
        batch._material_struct(stt_material().coefficients())


def test_oracle_dm_dcurrent_of_a_linear_field(small_box):
    import oracle
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    c = stt_material().coefficients(None)
    s = oracle.OracleSim(om, c, do_demag=False)
    x = small_box.points
    grad = np.array([[0.3, -0.1, 0.2], [0.05, 0.4, -0.3], [-0.2, 0.1, 0.15]])   # grad[c][d] = d m_c / d x_d
    m = np.array([1.0, 0.5, -0.4])[None, :] + x @ grad.T
    J = np.array([2e-3, -1e-3, 5e-4])
    s.set_stt(c["C4"], c["C5"], J)
    d = s.rhs(m).reshape(-1, 3)
    u = s.field("dm_dcurrent")
    assert np.abs(u - (grad @ J)[None, :]).max() < 1e-14
    s2 = oracle.OracleSim(om, c, do_demag=False)
    d0 = s2.rhs(m).reshape(-1, 3)
    mxu = np.cross(m, u)
    assert np.abs(d - (d0 + c["C4"] * np.cross(m, mxu) + c["C5"] * mxu)).max() < 1e-13 * np.abs(d).max()
