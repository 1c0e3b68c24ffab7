"""The oracle's BDF against an independent ODE solver on the full RHS.

scipy's DOP853 (an explicit 8th-order Runge-Kutta pair, nothing shared with
the oracle's CVODE restatement) integrates the oracle's own RHS (exchange,
FEM/BEM demag, LLG) of the plain-method configuration -- the 30 nm cube,
alpha 0.5, seeded m -- at rtol = atol = 1e-11, with Poisson solves at
1e-12.  The oracle's BDF must follow that solution at every 10 ps record:
within 5e-5 at the configuration's tolerance (1e-6, orders 1-2) and ten
times closer at 1e-8, so its errors shrink with its tolerance as a
convergent integrator's must.
"""
import numpy as np
import pytest

import oracle
from conftest import permalloy, seeded_m

scipy_integrate = pytest.importorskip("scipy.integrate")


def test_bdf_follows_dop853_on_the_plain_configuration(cube):
    om = oracle.OracleMesh(cube.points, cube.simplices)
    c = permalloy(0.5).coefficients("nmag")
    tight = dict(nbc=(1e-12, 1e-50, 5000), dbc=(1e-12, 1e-50, 5000), nthreads=1)
    s = oracle.OracleSim(om, c, **tight)
    m0 = seeded_m(om.n_nodes, seed=0, noise=0.01)
    times = [10.0 * k for k in range(1, 11)]   # 100 ps, simulation units of time (ps)
    sol = scipy_integrate.solve_ivp(lambda t, y: s.rhs(y.reshape(-1, 3)).copy(), (0.0, times[-1]),
                                    m0.reshape(-1), method="DOP853", rtol=1e-11, atol=1e-11, t_eval=times)
    assert sol.status == 0
    ref = sol.y.T.reshape(len(times), -1, 3)
    errs = {}
    for rt in (1e-6, 1e-8):
        b = oracle.OracleSim(om, c, **tight)
        b.ts_init(m0, rtol=rt, atol=rt, max_order=2)
        got = np.array([b.ts_advance(t)[1] for t in times])
        errs[rt] = np.abs(got - ref).max()
    print("max |m - DOP853| by BDF tolerance:", errs)
    assert errs[1e-6] <= 5e-5, errs
    assert errs[1e-8] <= 0.1 * errs[1e-6], errs
