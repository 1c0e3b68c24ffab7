"""The nmesh text reader and the structured mesher pinned to the
reference's own mesher.

tests/golden/cubicmesh/*.nmesh were written by utils/cubicmesh/cubicmesh.c,
compiled unmodified (oracle/Makefile, target ref-cubicmesh) and run by
tests/golden/make_ref_cubicmesh.py.  The reader must give the counts, the
volume and the face structure of a conforming box mesh; nmag.mesh.cubicmesh
must give the same simplices and regions and, printed as the mesher prints
them ("%f"), the same coordinates.  Where the reference tree is present the
mesher is built (oracle/_ref) and run live on further cases.
"""
import os

import numpy as np
import pytest

import oracle
from nmag import mesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cubicmesh")
CASES = {
    "box": ((4.0, 3.0, 2.0), (4, 3, 2), None),
    "slab_x": ((5.0, 2.0, 1.0), (4, 2, 1), "x:1.25,3.75"),
    "rod_z": ((1.0, 1.5, 2.5), (2, 3, 5), "z:0.5,1.5"),
    "offgrid_y": ((3.0, 3.0, 3.0), (3, 3, 3), "y:1.7"),
}


def _point_text(path):
    """The coordinate fields of an nmesh text file, as written."""
    with open(path) as f:
        rows = [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]
    n = int(rows[0][0])
    return [t for row in rows[1:1 + n] for t in row]


def _faces(simplices):
    f = np.concatenate([np.sort(simplices[:, [a, b, c]], axis=1)
                        for a, b, c in ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2))])
    _, counts = np.unique(f, axis=0, return_counts=True)
    return counts


def _check_same(m, path):
    ref = mesh.load_ascii(path)
    assert np.array_equal(m.simplices, ref.simplices)
    assert np.array_equal(m.regions, ref.regions)
    assert ["%f" % v for v in m.points.ravel()] == _point_text(path)


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_on_reference_mesher_files(name):
    sizes, nn, _ = CASES[name]
    path = os.path.join(GOLDEN, name + ".nmesh")
    with open(path) as f:
        f.readline()
        head = dict(kv.split(" = ") for kv in f.readline().lstrip("# ").strip().split(" \t"))
    m = mesh.load_ascii(path)
    nx, ny, nz = nn
    assert m.n_nodes == int(head["nodes"]) == (nx + 1) * (ny + 1) * (nz + 1)
    assert m.n_tets == int(head["simplices"]) == 6 * nx * ny * nz
    vol = m.tet_volumes()
    assert vol.min() > 0
    assert abs(vol.sum() - np.prod(sizes)) <= 1e-12 * np.prod(sizes)
    counts = _faces(m.simplices)   # conforming: inner faces twice, the box's surface once
    assert set(counts.tolist()) <= {1, 2}
    assert (counts == 1).sum() == 4 * (nx * ny + ny * nz + nx * nz)


@pytest.mark.parametrize("name", sorted(CASES))
def test_cubicmesh_equals_reference_files(name):
    sizes, nn, flt = CASES[name]
    _check_same(mesh.cubicmesh(sizes, nn, flt), os.path.join(GOLDEN, name + ".nmesh"))


def test_cubicmesh_regions_follow_the_filter():
    m = mesh.cubicmesh((5.0, 2.0, 1.0), (4, 2, 1), "x:1.25,3.75")
    cx = m.points[m.simplices].mean(axis=1)[:, 0]
    assert np.array_equal(m.regions, np.where(cx > 3.75, 3, np.where(cx > 1.25, 2, 1)))
    assert np.array_equal(mesh.cubicmesh((5.0, 2.0, 1.0), (4, 2, 1), (0, [1.25, 3.75])).regions, m.regions)
    assert np.array_equal(mesh.cubicmesh((5.0, 2.0, 1.0), (4, 2, 1), "0:1.25,3.75").regions, m.regions)


def test_cubicmesh_refuses_what_the_mesher_refuses():
    with pytest.raises(ValueError):
        mesh.cubicmesh((1.0, 1.0, 1.0), (0, 1, 1))
    with pytest.raises(ValueError):
        mesh.cubicmesh((1.0, -1.0, 1.0), (1, 1, 1))
    with pytest.raises(ValueError):
        mesh.cubicmesh((1.0, 1.0, 1.0), (1, 1, 1), "x:0.7,0.2")   # thresholds out of order
    with pytest.raises(ValueError):
        mesh.cubicmesh((1.0, 1.0, 1.0), (1, 1, 1), "w:0.5")


def test_cubicmesh_against_live_reference_mesher(tmp_path):
    if not oracle.build_ref_cubicmesh():
        pytest.skip("reference tree absent: the committed files pin the mesher instead")
    rng = np.random.default_rng(11)
    cases = [((7.3, 2.1, 0.9), (5, 3, 2), None), ((2.0, 2.0, 2.0), (4, 4, 4), "y:0.5,1.0,1.5"),
             ((10.0, 4.0, 3.0), (7, 3, 2), "x:2.9,6.1"), ((1.0, 1.0, 6.0), (1, 1, 9), "z:3.0")]
    for _ in range(3):
        sizes = tuple(float(v) for v in rng.uniform(0.5, 20.0, 3).round(3))
        cases.append((sizes, tuple(int(v) for v in rng.integers(1, 7, 3)), None))
    for k, (sizes, nn, flt) in enumerate(cases):
        path = oracle.ref_cubicmesh(str(tmp_path / ("m%d.nmesh" % k)), sizes, nn, flt)
        _check_same(mesh.cubicmesh(sizes, nn, flt), path)
