"""The oracle's BEM fill pinned to the reference's own code.

tests/golden/ref_bem.npz holds BEM matrices (whole, or sampled rows with the
whole matrix's row and column sums) filled by the reference's Lindholm stub,
src/bem3d_stubs.c:413-610, compiled unmodified against the project's caml
shim and driven as src/bem3d.ml:938-1047 drives it (made by
tests/golden/make_ref_bem.py).  The oracle restates that arithmetic in the
same operation order, so on one machine the two agree bit for bit: where the
reference tree is present the stub is built (oracle/_ref) and run live.
"""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_bem.npz")


def _mesh(args):
    from nmag import mesh
    nx, ny, nz = (int(a) for a in args[:3])
    return mesh.box_mesh(nx, ny, nz, *args[3:])


@pytest.mark.parametrize("name", ["box", "cube", "plate"])
def test_oracle_bem_equals_reference_fixture(name):
    g = np.load(GOLDEN)
    msh = _mesh(g[name + "_args"])
    om = oracle.OracleMesh(msh.points, msh.simplices)
    rows = g[name + "_rows"]
    # bit for bit on the machine that made the fixtures; elsewhere the host's
    # libm (log, acos) may round a last bit differently, hence 1e-15 of the
    # largest entry
    scale = np.abs(g[name + "_bem"]).max()
    assert np.abs(om.bem[rows] - g[name + "_bem"]).max() <= 1e-15 * scale
    assert np.abs(om.bem.sum(axis=1) - g[name + "_rowsum"]).max() <= 1e-13 * scale
    assert np.abs(om.bem.sum(axis=0) - g[name + "_colsum"]).max() <= 1e-13 * scale


def test_oracle_bem_equals_live_reference_stub():
    if not oracle.build_ref():
        pytest.skip("reference tree absent: the committed fixtures pin the fill instead")
    from nmag import mesh
    for msh in (mesh.cube_mesh(), mesh.box_mesh(7, 5, 4, 2.0, 3.0, 2.5), mesh.box_mesh(20, 6, 2, 2.5, 2.5, 1.5)):
        om = oracle.OracleMesh(msh.points, msh.simplices)
        assert np.array_equal(oracle.ref_bem(om), om.bem)
