"""The nmesh text reader's checks, as the reference's reader makes them
(src/mesh.ml:6619-6760): the tag and its major version, the summary line
whose counts place the sections, the number of entries per row, vertex
indices in range and distinct; and load()'s format dispatch
(nmeshlib/lib1.py:656-678,838-863).  Each case plants one defect in a file
written by save_ascii."""
import numpy as np
import pytest

from nmag import mesh


@pytest.fixture
def text(tmp_path):
    path = str(tmp_path / "m.nmesh")
    mesh.save_ascii(mesh.cubicmesh((2.0, 1.0, 1.0), (2, 1, 1), "x:1.0"), path)
    with open(path) as f:
        return path, f.read().splitlines()


def _write(path, lines):
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def test_round_trip_and_surfaces_skipped(text):
    path, lines = text
    m = mesh.cubicmesh((2.0, 1.0, 1.0), (2, 1, 1), "x:1.0")
    back = mesh.load_ascii(path)
    assert np.array_equal(back.points, m.points) and np.array_equal(back.simplices, m.simplices)
    assert np.array_equal(back.regions, m.regions)
    n, t = m.n_nodes, m.n_tets
    # two surface rows ("region1 region2 v0 v1 v2"), as the reference's writer may emit them
    lines = lines[:2] + lines[2:5 + n + t - 1] + ["2", " 1 -1 0 1 2", " 1 -1 0 2 3", "0"]
    lines[1] = lines[1].replace("surfaces = 0", "surfaces = 2")
    back = mesh.load_ascii(_write(path, lines))
    assert np.array_equal(back.simplices, m.simplices)


@pytest.mark.parametrize("edit, message", [
    (lambda L, n: ["# some other file"] + L[1:], "version of the file not given"),
    (lambda L, n: ["# PYFEM mesh file version 2.0"] + L[1:], "wrong version"),
    (lambda L, n: L[:1] + ["# nothing"] + L[2:], "mesh summary not given"),
    (lambda L, n: L[:3] + [" 0.0 0.0"] + L[4:], "LINE 4: Wrong number of point coordinates"),
    (lambda L, n: L[:4 + n] + [" 1 0 1 2"] + L[5 + n:], "LINE %d: Wrong number of simplex coordinates"),
    (lambda L, n: L[:4 + n] + [" 1 0 1 2 999"] + L[5 + n:], "LINE %d: Index 4 out of range"),
    (lambda L, n: L[:4 + n] + [" 1 0 1 1 2"] + L[5 + n:], "LINE %d: Duplicate index"),
    (lambda L, n: L[:4 + n] + [" a 0 1 2 3"] + L[5 + n:], "LINE %d: Wrong number of simplex region"),
    (lambda L, n: L[:4 + n + 3], "the file ends before the simplices"),
    (lambda L, n: L[:9], "LINE 10: the file ends before the points"),
])
def test_reader_refuses_what_the_reference_refuses(text, edit, message):
    path, lines = text
    n = 12   # nodes of the 2 x 1 x 1 mesh
    bad = _write(path, edit(lines, n))
    msg = message % (5 + n) if "%d" in message else message
    with pytest.raises(IOError, match=msg):
        mesh.load_ascii(bad)


def test_periodic_groups_are_refused(text):
    path, lines = text
    lines = list(lines)
    lines[1] = lines[1].replace("periodic = 0", "periodic = 1")
    lines[-1] = "1"
    lines.append("0 2")
    with pytest.raises(IOError, match="periodic"):
        mesh.load_ascii(_write(path, lines))


def test_load_dispatch(tmp_path, text):
    path, _ = text
    assert mesh.load(path).n_tets == 12
    h5path = str(tmp_path / "m.nmesh.h5")
    mesh.save_hdf5(mesh.load(path), h5path)
    assert mesh.load(h5path).n_tets == 12
    other = _write(str(tmp_path / "x.txt"), ["12", "0 0 0"])
    with pytest.raises(IOError, match="unknown file format"):
        mesh.load(other)
    with pytest.raises(IOError, match="does not exist"):
        mesh.load(str(tmp_path / "missing.nmesh"))
