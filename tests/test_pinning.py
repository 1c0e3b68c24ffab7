"""Pinning field (nmag_lam.py:417-436): the factor pin of every dm/dt term
and of the timestepper's Jacobian rows, on the oracle.  CPU only."""
import numpy as np

from conftest import permalloy, seeded_m


def test_oracle_pinning_scales_dmdt_and_jacobian_rows(small_box):
    import oracle
    c = permalloy(0.3).coefficients("nmag")
    om = oracle.OracleMesh(small_box.points, small_box.simplices, fill_bem=False)
    free = oracle.OracleSim(om, c, do_demag=False)
    pinned = oracle.OracleSim(om, c, do_demag=False)
    N = small_box.n_nodes
    pin = np.random.default_rng(31).choice([0.0, 1.0, 0.25], size=N)
    pinned.set_pinning(pin)
    m = seeded_m(N, seed=31, noise=0.5)
    for s in (free, pinned):
        s.set_h_ext([0.0, 0.02, 0.0])
    d_free = free.rhs(m).reshape(-1, 3)
    d_pin = pinned.rhs(m).reshape(-1, 3)
    assert np.abs(d_pin - pin[:, None] * d_free).max() <= 1e-15 * np.abs(d_free).max()
    assert np.all(d_pin[pin == 0.0] == 0.0)
    v = np.random.default_rng(32).standard_normal(3 * N)
    H = free.field("H_total")
    jf = free.jv(m, H, v).reshape(-1, 3)
    jp = pinned.jv(m, H, v).reshape(-1, 3)
    assert np.abs(jp - pin[:, None] * jf).max() <= 1e-15 * np.abs(jf).max()
