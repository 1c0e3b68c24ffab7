"""P1 point location and interpolation behind Simulation.probe_subfield
(main.py:1570-1700): a linear field is reproduced exactly inside the mesh,
points outside give None.  CPU only."""
import numpy as np

from nmag import mesh


def test_locate_and_interpolate_linear_field():
    msh = mesh.box_mesh(4, 3, 2, 2.0, 2.5, 1.5)
    A = np.array([[0.3, -0.2, 0.1], [0.05, 0.4, -0.3], [1.0, 0.0, 0.5]])
    vals = 0.7 + msh.points @ A.T             # (N, 3), linear in space
    rng = np.random.default_rng(5)
    lo, hi = msh.points.min(0), msh.points.max(0)
    for x in lo + (hi - lo) * rng.random((40, 3)):
        v = msh.interpolate(vals, x)
        assert np.allclose(v, 0.7 + A @ x, rtol=0, atol=1e-12)
        t, bary = msh.locate(x)
        assert abs(bary.sum() - 1.0) < 1e-12 and bary.min() >= -1e-10
        assert np.allclose(bary @ msh.points[msh.simplices[t]], x, atol=1e-12)
    # nodes and a scalar field
    s = msh.points[:, 0] * 2.0
    assert abs(msh.interpolate(s, msh.points[7]) - s[7]) < 1e-12
    assert msh.interpolate(vals, hi + 1.0) is None
    assert abs(msh.tet_volumes().sum() - np.prod(hi - lo)) < 1e-12
