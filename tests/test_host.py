"""Host-side tests (CPU): units, materials, meshes, the C-ABI library's
exports, and the product's independence from the oracle."""
import json
import os
import re

import numpy as np
import pytest

import nmag
from nmag import SI, mesh
from nmag import _build, _lib
from conftest import ROOT, permalloy

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "kat.json")))


def test_si_parsing_and_units():
    assert SI(1.0, "m/A s").dims == {"m": 1, "A": -1, "s": -1}
    assert SI(1.0, "J/m^3").dims == {"kg": 1, "m": -1, "s": -2}
    assert SI(2.0, "s^(-1)").dims == {"s": -1}
    su = nmag.simulation_units
    assert su.of(SI(8.6e5, "A/m")) == pytest.approx(0.86, rel=1e-15)
    assert su.of(SI(1e-12, "s")) == pytest.approx(1.0, rel=1e-15)
    assert su.of(SI(1e-9, "m")) == pytest.approx(1.0, rel=1e-15)
    assert su.of(nmag.si.mu0) == pytest.approx(GOLD["permalloy_alpha05"]["su_mu0"], rel=1e-15)
    with pytest.raises(ValueError):
        su.of(SI(1.0, "A/m"), compatible_with=SI("m"))


def test_material_coefficients_and_quirks():
    for key, alpha in (("permalloy_alpha05", 0.5), ("permalloy_alpha002", 0.02)):
        g = GOLD[key]
        c = permalloy(alpha).coefficients(None)
        assert c["C1"] == pytest.approx(g["C1"], rel=1e-14)
        assert c["C2"] == pytest.approx(g["C2"], rel=1e-14)
        q = permalloy(alpha).coefficients("nmag")
        # %g keeps 6 significant digits
        assert float("%g" % g["C1"]) == q["C1"]
        assert abs(q["C1"] / g["C1"] - 1) < 5e-6
    m = nmag.MagMaterial("x", do_precession=False)
    assert m.coefficients()["C1"] == 0.0
    # a polarisation switches the spin-transfer coefficients on
    stt = nmag.MagMaterial("stt", llg_polarisation=0.5).coefficients()
    assert stt["C4"] != 0.0 and stt["C5"] != 0.0


@pytest.mark.parametrize("n", [4, 8])
def test_box_mesh_counts(n):
    m = mesh.box_mesh(n, n, n, 2.0)
    g = GOLD["particles"][str(n)]
    assert m.n_nodes == g["nodes"] and m.n_tets == g["tets"]
    # every tet positively oriented volume h^3/6
    p = m.points[m.simplices]
    det = np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
    assert np.allclose(np.abs(det), 8.0)


def test_nmesh_ascii_round_trip(tmp_path, small_box):
    fn = str(tmp_path / "box.nmesh")
    mesh.save_ascii(small_box, fn)
    back = mesh.load_ascii(fn)
    assert np.array_equal(back.simplices, small_box.simplices)
    assert np.array_equal(back.regions, small_box.regions)
    assert np.array_equal(back.points, small_box.points)


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "nmag_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(nmg_\w+)\s*\(", txt, re.M)))


def test_exports_list_matches_header():
    assert sorted(_lib.EXPORTS) == header_symbols()


def test_library_builds_and_exports_every_symbol():
    path = _build.build()
    import ctypes
    L = ctypes.CDLL(path)
    for name in header_symbols():
        assert hasattr(L, name), name
    assert L.nmg_version() == 10000


def test_create_rejects_bad_input_without_gpu():
    # argument checks run before any CUDA call
    L = _lib.lib()
    import ctypes as C
    mt = _lib.Material()
    h = C.c_void_p()
    pts = np.zeros(12)
    bad = np.array([0, 1, 2, 7], dtype=np.int32)
    rc = L.nmg_create(pts, 4, bad, 1, C.byref(mt), None, C.byref(h))
    assert rc == -3
    assert b"missing node" in L.nmg_last_error(None)


def test_create_rejects_bad_anchor_options_without_gpu():
    # the anchored product's tolerance: finite, non-negative, compensated form only
    L = _lib.lib()
    import ctypes as C
    mt = _lib.Material()
    mt.Ms = 1.0
    h = C.c_void_p()
    pts = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)
    tet = np.array([0, 1, 2, 3], dtype=np.int32)
    for prec, tol, msg in ((2, -1.0, b"finite and non-negative"), (2, float("nan"), b"finite and non-negative"),
                           (0, 1e-3, b"compensated product"), (1, 1e-3, b"compensated product")):
        op = _lib.Options()
        op.do_demag = 1
        op.bem_precision = prec
        op.bem_anchor_tol = tol
        rc = L.nmg_create(pts, 4, tet, 1, C.byref(mt), C.byref(op), C.byref(h))
        assert rc == -6, (prec, tol, rc)
        assert msg in L.nmg_last_error(None), L.nmg_last_error(None)


def test_jacobian_option_checks_without_gpu():
    # the Newton matrix's Jacobian: three named levels, a Poisson tolerance in (0, 1)
    import nmag
    from nmag.simulation import JACOBIAN_LEVELS
    assert JACOBIAN_LEVELS == ("approximate", "local", "exact")
    for bad in ({"jacobian": "full"}, {"jacobian_demag_rtol": 0.0}, {"jacobian_demag_rtol": 1.5}):
        with pytest.raises(ValueError):
            nmag.Simulation("j", **bad)
    sim = nmag.Simulation("j", jacobian="exact", jacobian_demag_rtol=1e-6)
    assert (sim.jacobian, sim.jacobian_demag_rtol) == ("exact", 1e-6)
    L = _lib.lib()
    assert L.nmg_set_jacobian(None, 2, 1e-6) == -1
    assert L.nmg_jacobian_apply(None, None, None, None) == -1


def test_batch_rejects_bad_integrator_without_gpu():
    import ctypes as C
    L = _lib.lib()
    pts = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)
    tet = np.array([0, 1, 2, 3], dtype=np.int32)
    part = (_lib.Particle * 1)()
    part[0].coords = pts.ctypes.data
    part[0].n_nodes = 4
    part[0].tets = tet.ctypes.data
    part[0].n_tets = 1
    o = _lib.BatchOptions()
    o.n_stages, o.cg_maxits, o.cg_rtol = 1, 10, 1e-6
    o.integrator = 2
    b = C.c_void_p()
    rc = L.nmg_batch_create(part, 1, C.byref(o), C.byref(b))
    assert rc == -2
    assert b"integrator" in L.nmg_batch_last_error(None)


def test_product_does_not_import_oracle():
    pkg = os.path.join(ROOT, "nmag-src_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".h")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in txt and "liboracle" not in txt, f


def _shelled_box():
    """A 6x6x4 box whose outer layer of cells is vacuum (region 0): the
    magnetic part is the inner 4x4x2 box."""
    from nmag import mesh
    outer = mesh.box_mesh(6, 6, 4, 2.0)
    cen = outer.points[outer.simplices].mean(axis=1)
    inside = np.all((cen > 2.0) & (cen < np.array([10.0, 10.0, 6.0])), axis=1)
    return mesh.Mesh(outer.points, outer.simplices, np.where(inside, 1, 0))


def test_magnetic_part_drops_vacuum():
    from nmag import mesh
    shelled = _shelled_box()
    part, node_map = mesh.magnetic_part(shelled)
    inner = mesh.box_mesh(4, 4, 2, 2.0, origin=(2.0, 2.0, 2.0))
    assert part.n_nodes == inner.n_nodes and part.n_tets == inner.n_tets
    assert (part.regions == 1).all()
    np.testing.assert_array_equal(part.points, shelled.points[node_map])
    # same tetrahedra (as coordinate sets) as the inner box built directly
    key = lambda m: sorted(tuple(sorted(map(tuple, np.round(m.points[t], 9)))) for t in m.simplices)
    assert key(part) == key(inner)


def test_load_mesh_region_checks_without_gpu():
    import nmag
    from nmag import SI
    shelled = _shelled_box()
    a = nmag.MagMaterial("A", Ms=SI(8e5, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"))
    b = nmag.MagMaterial("B", Ms=SI(1e6, "A/m"), exchange_coupling=SI(1.3e-11, "J/m"))
    sim = nmag.Simulation("regions")
    # two materials are fine (one m each), but this mesh has one magnetic region
    with pytest.raises(ValueError):
        sim.load_mesh(shelled, [("a", a), ("b", b)], unit_length=SI(1e-9, "m"))
    two = nmag.mesh.Mesh(shelled.points, shelled.simplices, np.where(shelled.regions == 1, 2, 1))
    with pytest.raises(ValueError):
        sim.load_mesh(two, [("a", a)], unit_length=SI(1e-9, "m"))
    # one (region, materials) pair per region of the mesh (main.py:1174-1180)
    with pytest.raises(ValueError):
        sim.load_mesh(two, [("a", a), ("b", a), ("c", a)], unit_length=SI(1e-9, "m"))


def test_si_physical_interface():
    """si_units/lib.py: in_units_of, get_units, comparisons (zero against any
    dimension), abs, str."""
    from nmag import SI
    d = SI(10.0, "m")
    assert d.in_units_of(SI(2.54e-2, "m")) == pytest.approx(393.7007874015748)
    with pytest.raises(ValueError):
        d.in_units_of(SI(1.0, "s"))
    assert d.get_units().value == 1.0 and d.get_units().dims == d.dims
    assert SI(1.0, "m") < SI(2.0, "m") and SI(3.0, "m") >= SI(3.0, "m") and SI(0.0, "s") < SI(1.0, "m")
    with pytest.raises(ValueError):
        SI(1.0, "m") < SI(2.0, "s")
    assert SI(2.0, "A/m") == SI(2.0, "A/m") and SI(2.0, "A/m") != SI(2.0, "m")
    assert abs(SI(-3.0, "s")).value == 3.0
    assert str(SI(1e6, "A/m")) == "<SI: 1e+06  A / m >"
    import nmag
    assert nmag.never.match_time({"step": 0}) is False


def test_str_of_si_vector():
    """The expectations of si_units/test_lib.py."""
    from nmag.si import SI, str_of_SI_vector
    H = [SI(1000000, ["m", -1.0, "A", 1.0]), SI(0, ["m", -1.0, "A", 1.0]), SI(0, ["m", -1.0, "A", 1.0])]
    assert str_of_SI_vector([SI(0, "A/m"), SI(100, "A/m")]) == "[0 100]<A/m>"
    assert str_of_SI_vector([0, SI(123, "A/m")]) == "[0 123]<A/m>"
    assert str_of_SI_vector([0, SI(123, "A/m"), 0]) == "[0 123 0]<A/m>"
    assert str_of_SI_vector(H) == "[1e+06 0 0]<A/m>"
    assert str_of_SI_vector([SI(1, "A/m")]) == "[1]<A/m>"
    assert str_of_SI_vector(None) == "None"
