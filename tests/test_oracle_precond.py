"""The Newton systems' preconditioner: the device's block-Jacobi form
against the reference's own form, both in the oracle's BDF.

The reference preconditions CVODE's GMRES with P = I - gamma J assembled
and solved by PETSc GMRES + bjacobi/ILU(0) to pc_rtol = 1e-2, pc_atol = 1e-7
(nsim.ml:2210-2262,2419-2483; main.py:720-739).  The device inverts each
node's 3x3 block of P exactly (one block-Jacobi sweep).  The oracle restates
both (om_bdf_set_precond); these tests check that the assembled matrix is
the Newton matrix of the Jacobian-vector product and that on the
plain-method configuration (30 nm cube, alpha 0.5, rtol = atol = 1e-6, 1 ns,
m(t) every 10 ps) the two preconditioners give the same trajectory to the
metric's 1e-4 and nearly the same steps; only the Krylov work differs.
"""
import numpy as np
import pytest

import oracle
from conftest import permalloy, seeded_m


@pytest.fixture(scope="module")
def ocube(cube):
    return oracle.OracleMesh(cube.points, cube.simplices)


def test_assembled_newton_matrix_is_the_jacobian_product(small_box):
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    s = oracle.OracleSim(om, permalloy(0.3).coefficients("nmag"), do_demag=False)
    rng = np.random.default_rng(5)
    mJ = seeded_m(om.n_nodes, seed=1, noise=0.5)
    HJ = rng.standard_normal((om.n_nodes, 3))
    for pin in (None, (rng.random(om.n_nodes) > 0.3).astype(np.float64)):
        if pin is not None:
            s.set_pinning(pin)
        for gamma in (0.0, 1e-3, 0.7):
            v = rng.standard_normal(3 * om.n_nodes)
            ref = v - gamma * s.jv(mJ, HJ, v)
            got = s.pc_matrix_apply(mJ, HJ, gamma, v)
            assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


def test_reference_preconditioner_on_the_plain_configuration(ocube):
    c = permalloy(0.5).coefficients("nmag")
    m0 = seeded_m(ocube.n_nodes, seed=0, noise=0.01)
    runs = {}
    for pc in ("block", "reference"):
        s = oracle.OracleSim(ocube, c, nthreads=1)   # one thread: a fixed summation order
        s.ts_init(m0, rtol=1e-6, atol=1e-6, precond=pc)
        rec = np.array([s.ts_advance(10.0 * k)[1] for k in range(1, 101)])
        runs[pc] = (rec, s.ts_stats())
    (mb, sb), (mr, sr) = runs["block"], runs["reference"]
    assert np.abs(mb - mr).max() <= 1e-4
    assert abs(sb["nst"] - sr["nst"]) <= 0.05 * sr["nst"]
    assert sr["pc_iterations"] > 0 and sb["pc_iterations"] == 0
    # the stronger preconditioner needs fewer outer Krylov iterations per Newton iteration
    assert sr["nli"] / sr["nni"] < sb["nli"] / sb["nni"]
