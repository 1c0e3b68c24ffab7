"""The dense torch reference of the differentiation form, checked on CPU
against the C oracle: with uniform element weights it must reproduce the
oracle's RHS (H_eff and dm/dt) and the oracle's fixed-step RK4."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from conftest import permalloy, seeded_m  # noqa: E402
from dense_llg import DenseLLG  # noqa: E402


def _material(K1=0.0):
    import nmag
    from nmag import SI
    mat = permalloy(0.5)
    if K1:
        mat = nmag.MagMaterial("Py", Ms=SI(8.6e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"), llg_damping=0.5,
                               llg_gamma_G=SI(2.211e5, "m/A s"),
                               anisotropy=nmag.uniaxial_anisotropy(axis=[0.3, 0.4, 0.866], K1=SI(K1, "J/m^3")))
    return mat


def _setup(msh, K1):
    mat = _material(K1)
    c = mat.coefficients("nmag")
    om = oracle.OracleMesh(msh.points, msh.simplices)
    sim = oracle.OracleSim(om, c, nbc=(1e-13, 1e-50, 20000), dbc=(1e-13, 1e-50, 20000))
    dense = DenseLLG(msh.points, msh.simplices, om.bem, om.node_of_b, c, axis=c["axis"])
    T = len(msh.simplices)
    one = torch.ones(T, dtype=torch.float64)
    kappa = torch.full((T,), c["anis_coeff"], dtype=torch.float64)
    return c, sim, dense, (one, one, kappa)


@pytest.mark.parametrize("K1", [0.0, 5e5])
def test_dense_rhs_matches_oracle(small_box, K1):
    c, sim, dense, (wK, wD, kappa) = _setup(small_box, K1)
    N = len(small_box.points)
    m = seeded_m(N, seed=5, noise=0.3)
    hext = np.array([0.01, -0.02, 0.005])
    sim.set_h_ext(hext)
    f_or = sim.rhs(m).reshape(N, 3)
    H_or = sim.field("H_total")
    ops = dense.operators(wK, wD, kappa)
    he = torch.as_tensor(np.broadcast_to(hext, (N, 3)).copy())
    f_d, H_d = dense.rhs(torch.as_tensor(m), ops, he)
    assert np.abs(H_d.numpy() - H_or).max() <= 1e-9 * np.abs(H_or).max()
    assert np.abs(f_d.numpy() - f_or).max() <= 1e-9 * np.abs(f_or).max()


def test_dense_rk4_matches_oracle(small_box):
    c, sim, dense, (wK, wD, kappa) = _setup(small_box, 0.0)
    N = len(small_box.points)
    m0 = seeded_m(N, seed=6, noise=0.3)
    sim.set_h_ext(np.zeros(3))
    m_or = sim.rk4(m0.copy(), 0.05, 10).reshape(-1)
    mT, hist = dense.trajectory(torch.as_tensor(m0.reshape(-1)), wK, wD, kappa, torch.zeros(0, dtype=torch.float64),
                                torch.zeros(N, 3, dtype=torch.float64), 0.05, 10, 1)
    assert np.abs(mT.numpy() - m_or).max() <= 1e-10
    assert hist.shape == (10, 3)
