"""Differentiation form on the GPU: the CUDA RK4 trajectory with per-element
parameters and its hand-written discrete adjoint (nmg_rk4_forward /
nmg_rk4_adjoint via nmag.adjoint.RK4Trajectory), checked against
  * the plain RK4 entry point (uniform weights),
  * a dense FP64 torch autograd reference on the 1331-node cube, and
  * central finite differences (h = 1e-6 relative) along seeded directions.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle  # noqa: E402
from conftest import permalloy, seeded_m  # noqa: E402
from dense_llg import DenseLLG  # noqa: E402
from test_gpu_parity import make_engine  # noqa: E402

pytestmark = pytest.mark.gpu

DT = 0.1          # 0.1 ps in simulation units


def _mu0_su():
    from nmag.si import simulation_units
    from nmag import si
    return simulation_units.of(si.mu0)


def _params(T, n_pulses, seed_ms=3, seed_p=4):
    """Per-element Ms (su) 0.86 (1 + 0.05 N(0,1)), K1 = 0, pulses N(0, 5 mT)/mu0 (su)."""
    rng = np.random.default_rng(seed_ms)
    Ms_T = 0.86 * (1.0 + 0.05 * rng.standard_normal(T))
    K1_T = np.zeros(T)
    rng = np.random.default_rng(seed_p)
    pulses = rng.standard_normal((n_pulses, 3)) * (5e-3 / (4e-7 * np.pi)) * 1e-6   # A/m -> su (1e-3 A / 1e-9 m)
    return Ms_T, K1_T, pulses


@pytest.fixture(scope="module")
def cube_setup(cube):
    mat = permalloy(0.5)
    eng = make_engine(cube, mat, tol=1e-12)
    c = mat.coefficients("nmag")
    return eng, c, cube


def _cuda(x):
    return torch.as_tensor(np.ascontiguousarray(x, np.float64)).cuda()


def _run(eng, c, m0, Ms_T, K1_T, pulses, nsteps, ckpt, spp, axis=(1.0, 0.0, 0.0), grad=True):
    from nmag import adjoint
    tM = _cuda(Ms_T).requires_grad_(grad)
    tK = _cuda(K1_T).requires_grad_(grad)
    tP = _cuda(pulses).requires_grad_(grad)
    tm = _cuda(m0.reshape(-1)).requires_grad_(grad)
    mT, hist = adjoint.rk4_trajectory(eng, tm, tM, tK, tP, axis, c["Ms"], _mu0_su(), DT, nsteps, ckpt, spp)
    loss = adjoint.film_loss(hist)
    if not grad:
        return loss.item(), mT.detach().cpu().numpy(), hist.detach().cpu().numpy()
    loss.backward()
    return (loss.item(), tm.grad.cpu().numpy(), tM.grad.cpu().numpy(), tK.grad.cpu().numpy(),
            tP.grad.cpu().numpy(), hist.detach().cpu().numpy())


def test_uniform_weights_match_plain_rk4(cube_setup):
    eng, c, cube = cube_setup
    N, T = len(cube.points), len(cube.simplices)
    m0 = seeded_m(N, seed=0)
    eng.set_h_ext(np.zeros(3))
    d = _cuda(m0.reshape(-1))
    eng.clear_element_params()
    eng.rk4_device(int(d.data_ptr()), DT, 6)
    torch.cuda.synchronize()
    plain = d.cpu().numpy()
    _, mT, _ = _run(eng, c, m0, np.full(T, c["Ms"]), np.zeros(T), np.zeros((0, 3)), 6, 2, 1, grad=False)
    eng.clear_element_params()
    assert np.abs(mT - plain).max() <= 1e-10


def test_adjoint_matches_dense_autograd(cube_setup):
    _check_dense(*cube_setup)


def test_adjoint_matches_dense_autograd_compensated(cube):
    """Compensated BEM form: forward product and its transpose in FP32 +
    BF16 pairs (the adjoint differentiates the same map); same bounds."""
    mat = permalloy(0.5)
    eng = make_engine(cube, mat, tol=1e-12, bem_precision=2)
    _check_dense(eng, mat.coefficients("nmag"), cube)
    eng.close()


def test_adjoint_matches_dense_autograd_mixed_backward_cg(cube):
    """The backward pass's Poisson solves by the mixed-precision CG (FP64
    residual refinement to 1e-12): same bounds."""
    from test_gpu_ensemble import make_ensemble
    mat = permalloy(0.5)
    eng, _ = make_ensemble(cube, mat, 1, bem_precision=2, adjoint_cg=1)
    _check_dense(eng, mat.coefficients("nmag"), cube)
    eng.close()


def _check_dense(eng, c, cube):
    N, T = len(cube.points), len(cube.simplices)
    nsteps, ckpt, spp, npul = 12, 5, 3, 4
    m0 = seeded_m(N, seed=0)
    Ms_T, K1_T, pulses = _params(T, npul)
    K1_T = 0.05 * np.random.default_rng(9).standard_normal(T)   # nonzero anisotropy exercises its adjoint
    eng.set_h_ext(np.zeros(3))
    loss, g_m0, g_Ms, g_K1, g_P, hist = _run(eng, c, m0, Ms_T, K1_T, pulses, nsteps, ckpt, spp)
    eng.clear_element_params()
    # dense FP64 autograd reference
    from nmag import adjoint
    om = oracle.OracleMesh(cube.points, cube.simplices)
    dense = DenseLLG(cube.points, cube.simplices, om.bem, om.node_of_b, c, axis=(1.0, 0.0, 0.0))
    tm = torch.as_tensor(m0.reshape(-1).copy()).requires_grad_(True)
    tM = torch.as_tensor(Ms_T).requires_grad_(True)
    tK = torch.as_tensor(K1_T).requires_grad_(True)
    tP = torch.as_tensor(pulses).requires_grad_(True)
    wK, wD, kap = adjoint.element_weights(tM, tK, c["Ms"], _mu0_su())
    _, hd = dense.trajectory(tm, wK, wD, kap, tP, torch.zeros(N, 3, dtype=torch.float64), DT, nsteps, spp)
    ld = adjoint.film_loss(hd)
    ld.backward()
    assert abs(loss - ld.item()) <= 1e-10 * abs(ld.item())
    assert np.abs(hist - hd.detach().numpy()).max() <= 1e-10

    def rel(a, b):
        return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
    assert rel(g_m0, tm.grad.numpy()) <= 1e-7
    assert rel(g_Ms, tM.grad.numpy()) <= 1e-7
    assert rel(g_K1, tK.grad.numpy()) <= 1e-7
    assert rel(g_P, tP.grad.numpy()) <= 1e-7


def test_adjoint_matches_finite_differences(cube_setup):
    eng, c, cube = cube_setup
    N, T = len(cube.points), len(cube.simplices)
    nsteps, ckpt, spp, npul = 10, 4, 2, 5
    m0 = seeded_m(N, seed=0)
    Ms_T, K1_T, pulses = _params(T, npul)
    eng.set_h_ext(np.zeros(3))
    loss, _, g_Ms, g_K1, g_P, _ = _run(eng, c, m0, Ms_T, K1_T, pulses, nsteps, ckpt, spp)
    h = 1e-6
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(8):
        dM = Ms_T * rng.standard_normal(T)           # relative perturbation of Ms
        dK = 0.05 * rng.standard_normal(T)           # K1 starts at 0: absolute scale 0.05 su (5e4 J/m^3)
        dP = np.abs(pulses).mean() * rng.standard_normal(pulses.shape)
        lp = _run(eng, c, m0, Ms_T + h * dM, K1_T + h * dK, pulses + h * dP, nsteps, ckpt, spp, grad=False)[0]
        lm = _run(eng, c, m0, Ms_T - h * dM, K1_T - h * dK, pulses - h * dP, nsteps, ckpt, spp, grad=False)[0]
        fd = (lp - lm) / (2 * h)
        ad = g_Ms @ dM + g_K1 @ dK + (g_P * dP).sum()
        worst = max(worst, abs(fd - ad) / max(abs(ad), 1e-30))
    eng.clear_element_params()
    assert worst <= 1e-5, worst
