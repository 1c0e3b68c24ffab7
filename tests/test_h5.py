"""The HDF5 reader and writer (nmag/h5.py) and the nmesh HDF5 mesh files.

No HDF5 library is installed, and the reference tree holds no HDF5 file.
The one file on the machine that the HDF5 library wrote (a MATLAB 7.3 file
in scipy's test data) pins the reader's core structures; otherwise these
tests check the module against itself: files written by the
writer (every layout, filter, datatype and group size it produces) read
back exactly, hand-assembled structures the writer does not produce (a
version 2 object header with compact links, version 1/2 layout and
version 2 filter-pipeline messages, version 3 attributes) parse as the
format specification lays them out, and the mesh layout of
nfem/hdf5_v01.py:1370-1545 (tags in /etc, /mesh/points, /mesh/simplices,
/mesh/simplicesregions) round-trips through load / save.
"""
import os
import struct
import zlib

import numpy as np
import pytest

from nmag import h5, mesh


def test_writer_reader_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    data = {
        "/a/f64": rng.standard_normal((37, 3)),
        "/a/f32": rng.standard_normal(11).astype(np.float32),
        "/a/i32": rng.integers(-1000, 1000, (5, 4)).astype(np.int32),
        "/a/u8": np.arange(200, dtype=np.uint8),
        "/a/i64_3d": rng.integers(0, 1 << 40, (2, 3, 4)),
        "/b/scalar": np.float64(2.5),
        "/b/strings": np.array([b"nmesh", b"1.0"]),
        "/b/empty": np.zeros((0, 3)),
        "/c/d/e/deep": np.arange(7, dtype=np.int32),
    }
    w = h5.Writer()
    for path, arr in data.items():
        w.create_dataset(path, arr)
    big = rng.standard_normal((1000, 3))
    w.create_dataset("/chunked/deflate", big, chunks=(100, 3), compression=6)
    w.create_dataset("/chunked/shuffle", big, chunks=(128, 2), shuffle=True, compression=1)
    w.create_dataset("/chunked/plain", big[:, 0].copy(), chunks=(33,))
    tab = np.zeros(4, dtype=[("t", "<f8"), ("step", "<i4"), ("m", "<f8", (3,)), ("name", "S6")])
    tab["t"], tab["step"] = [0.0, 1e-12, 2e-12, 3e-12], [0, 5, 10, 15]
    tab["m"] = rng.standard_normal((4, 3))
    tab["name"] = [b"a", b"bb", b"ccc", b"dddd"]
    w.create_dataset("/table", tab)
    for k in range(40):   # several symbol-table nodes in one group
        w.create_dataset("/many/x%03d" % k, np.full(2, k, np.int32))
    w.set_attrs("/", {"TITLE": "root title", "VERSION": "1.0"})
    w.set_attrs("/a/f64", {"CLASS": "ARRAY", "scale": np.array([1.5, 2.5]), "n": np.int32(7)})
    path = str(tmp_path / "t.h5")
    w.save(path)

    assert h5.is_hdf5(path)
    f = h5.File(path)
    assert f.keys() == ["a", "b", "c", "chunked", "many", "table"]
    for p, arr in data.items():
        got = f[p].read()
        assert got.shape == np.shape(arr) and got.dtype == np.asarray(arr).dtype, p
        assert np.array_equal(got, arr), p
    assert np.array_equal(f["/chunked/deflate"].read(), big)
    assert np.array_equal(f["/chunked/shuffle"].read(), big)
    assert np.array_equal(f["/chunked/plain"].read(), big[:, 0])
    t = f["/table"].read()
    for name in tab.dtype.names:
        assert np.array_equal(t[name], tab[name]), name
    assert f["many"].keys() == ["x%03d" % k for k in range(40)]
    assert np.array_equal(f["/many/x039"].read(), [39, 39])
    assert f.attrs["TITLE"] == "root title"
    a = f["/a/f64"].attrs
    assert a["CLASS"] == "ARRAY" and np.array_equal(a["scale"], [1.5, 2.5]) and a["n"] == 7
    with pytest.raises(KeyError):
        f["/a/missing"]


def _ohdr_v2(msgs):
    """A version 2 object header (no times, 1-byte chunk size; checksum bytes zero)."""
    body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)
    return b"OHDR" + bytes([2, 0, len(body)]) + body + b"\0" * 4


def test_reader_structures_the_writer_does_not_produce():
    """A version 2 superblock whose root is a version 2 object header with
    compact link messages to (1) a dataset with a version 1 layout and a
    version 2 filter pipeline (deflate) over two chunks, and (2) a dataset
    with a version 2 compact layout and a version 3 attribute."""
    arr = np.arange(12, dtype="<f8").reshape(6, 2)
    c0, c1 = zlib.compress(arr[:3].tobytes()), zlib.compress(arr[3:].tobytes())
    out = bytearray(48)   # superblock v2 (filled in below)

    def put(b):
        while len(out) % 8:
            out.append(0)
        at = len(out)
        out.extend(b)
        return at

    a0, a1 = put(c0), put(c1)
    tree = b"TREE" + bytes([1, 0]) + struct.pack("<H", 2) + struct.pack("<QQ", h5.UNDEF, h5.UNDEF)
    for off, at, n in ((0, a0, len(c0)), (3, a1, len(c1))):
        tree += struct.pack("<II", n, 0) + struct.pack("<QQQ", off, 0, 0) + struct.pack("<Q", at)
    tree += struct.pack("<II", 0, 0) + struct.pack("<QQQ", 6, 2, 0)
    bt = put(tree)
    f64 = h5._dt_msg(np.dtype("<f8"))
    space_v2 = struct.pack("<BBBB", 2, 2, 0, 1) + struct.pack("<QQ", 6, 2)
    layout_v1 = struct.pack("<BBB5x", 1, 3, 2) + struct.pack("<Q", bt) + struct.pack("<III", 3, 2, 8)
    pipeline_v2 = struct.pack("<BB", 2, 1) + struct.pack("<HHH", 1, 0, 1) + struct.pack("<I", 4)
    d1 = put(_ohdr_v2([(1, space_v2), (3, f64), (8, layout_v1), (11, pipeline_v2)]))
    vals = np.array([7, 8, 9], dtype="<i4")
    i32 = h5._dt_msg(np.dtype("<i4"))
    space1 = struct.pack("<BBBB", 2, 1, 0, 1) + struct.pack("<Q", 3)
    layout_c = struct.pack("<BBH", 3, 0, vals.nbytes) + vals.tobytes()
    sdt = bytes([0x13, 0, 0, 0]) + struct.pack("<I", 5)
    attr_v3 = struct.pack("<BBHHHB", 3, 0, 6, len(sdt), 4, 0) + b"TITLE\0" + sdt + \
        struct.pack("<BBBB", 2, 0, 0, 0) + b"hello"
    # an enumeration attribute (read as its base integer) and a variable-length
    # string attribute (outside the subset: skipped, the rest still read)
    u8 = h5._dt_msg(np.dtype("u1"))
    enum = bytes([0x18]) + (2).to_bytes(3, "little") + struct.pack("<I", 1) + u8 + \
        b"OFF\0\0\0\0\0" + b"ON\0\0\0\0\0\0" + bytes([0, 1])
    attr_enum = struct.pack("<BBHHHB", 3, 0, 5, len(enum), 4, 0) + b"FLAG\0" + enum + \
        struct.pack("<BBBB", 2, 0, 0, 0) + bytes([1])
    vl = bytes([0x19, 1, 0, 0]) + struct.pack("<I", 16) + u8
    attr_vl = struct.pack("<BBHHHB", 3, 0, 3, len(vl), 4, 0) + b"VL\0" + vl + \
        struct.pack("<BBBB", 2, 0, 0, 0) + b"\0" * 16
    d2 = put(_ohdr_v2([(1, space1), (3, i32), (8, layout_c), (12, attr_v3), (12, attr_enum), (12, attr_vl)]))

    def link(name, addr):
        nm = name.encode()
        return struct.pack("<BB", 1, 0) + bytes([len(nm)]) + nm + struct.pack("<Q", addr)

    root = put(_ohdr_v2([(6, link("chunked", d1)), (6, link("compact", d2))]))
    sb = h5.SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, h5.UNDEF, len(out), root) + b"\0" * 4
    out[0:48] = sb
    f = h5.File(bytes(out))
    assert f.keys() == ["chunked", "compact"]
    assert np.array_equal(f["chunked"].read(), arr)
    assert np.array_equal(f["compact"].read(), vals)
    assert f["compact"].attrs["TITLE"] == "hello"
    assert f["compact"].attrs["FLAG"] == 1 and "VL" not in f["compact"].attrs


def test_nmesh_hdf5_round_trip_and_dispatch(tmp_path):
    m = mesh.box_mesh(4, 3, 2, 2.0, 2.5, 1.5)
    m.regions[:5] = 2
    path = str(tmp_path / "box.nmesh.h5")
    mesh.save_hdf5(m, path, sifactor=1e-9, unit="<SI: 1e-09 m >")
    r = mesh.load(path)   # recognised by its signature
    assert np.array_equal(r.points, m.points)
    assert np.array_equal(r.simplices, m.simplices) and r.simplices.dtype == np.int32
    assert np.array_equal(r.regions, m.regions)
    assert r.sifactor == 1e-9
    f = h5.File(path)
    assert mesh._tag(f, "filetype") == "nmesh" and mesh._tag(f, "fileversion") == "1.0"
    assert f["/mesh/points"].attrs["CLASS"] == "CARRAY"
    # the ASCII file of the same mesh reads the same
    apath = str(tmp_path / "box.nmesh")
    mesh.save_ascii(m, apath)
    a = mesh.load(apath)
    assert np.array_equal(a.points, r.points) and np.array_equal(a.simplices, r.simplices)


def test_nmesh_hdf5_refuses_other_files(tmp_path):
    w = h5.Writer()
    w.create_dataset("/etc/filetype", np.array([b"other"]))
    w.create_dataset("/etc/fileversion", np.array([b"1.0"]))
    w.create_dataset("/mesh/points", np.zeros((4, 3)))
    path = str(tmp_path / "x.h5")
    w.save(path)
    with pytest.raises(IOError):
        mesh.load_hdf5(path)
    w2 = h5.Writer()
    w2.create_dataset("/etc/filetype", np.array([b"nmesh"]))
    w2.create_dataset("/etc/fileversion", np.array([b"1.0"]))
    w2.create_dataset("/mesh/points", np.zeros((4, 3)))
    w2.save(path)
    with pytest.raises(IOError):   # simplices missing
        mesh.load_hdf5(path)
    with open(path, "wb") as fh:
        fh.write(b"not hdf5 at all")
    with pytest.raises(h5.HDF5Error):
        h5.File(path)


def test_simulation_save_mesh_by_extension(tmp_path):
    import nmag
    sim = nmag.Simulation("sm")
    sim.mesh = mesh.box_mesh(2, 2, 2, 1.0)
    sim.save_mesh(str(tmp_path / "m.nmesh.h5"))
    sim.save_mesh(str(tmp_path / "m.nmesh"))
    a, b = mesh.load(str(tmp_path / "m.nmesh.h5")), mesh.load(str(tmp_path / "m.nmesh"))
    assert np.array_equal(a.simplices, b.simplices) and np.allclose(a.points, b.points)
    assert os.path.getsize(str(tmp_path / "m.nmesh.h5")) > 96


def test_reader_two_level_chunk_btree(tmp_path):
    """A chunked dataset whose chunk index has an internal node over two
    leaves (the form larger PyTables arrays take): every chunk is found."""
    arr = np.arange(40, dtype="<i4").reshape(10, 4)
    w = h5.Writer()
    w.create_dataset("/d", arr, chunks=(3, 4))   # 4 chunks in one leaf; the leaf is split below
    path = str(tmp_path / "c.h5")
    w.save(path)
    raw = bytearray(open(path, "rb").read())
    f = h5.File(bytes(raw))
    b = f.b
    p, _ = f["d"]._msg(0x08)
    leaf = b.addr(p + 3)
    ksize = 8 + 8 * 3
    keys = [(raw[leaf + 24 + k * (ksize + 8): leaf + 24 + k * (ksize + 8) + ksize],
             raw[leaf + 24 + k * (ksize + 8) + ksize: leaf + 24 + (k + 1) * (ksize + 8)]) for k in range(4)]
    last = raw[leaf + 24 + 4 * (ksize + 8): leaf + 24 + 4 * (ksize + 8) + ksize]

    def node(level, entries, final):
        t = b"TREE" + bytes([1, level]) + struct.pack("<H", len(entries)) + struct.pack("<QQ", h5.UNDEF, h5.UNDEF)
        for key, child in entries:
            t += bytes(key) + bytes(child)
        return t + bytes(final)

    def put(blob):
        while len(raw) % 8:
            raw.append(0)
        at = len(raw)
        raw.extend(blob)
        return at

    l0 = put(node(0, keys[:2], keys[2][0]))
    l1 = put(node(0, keys[2:], last))
    root = put(node(1, [(keys[0][0], struct.pack("<Q", l0)), (keys[2][0], struct.pack("<Q", l1))], last))
    raw[p + 3:p + 11] = struct.pack("<Q", root)
    assert np.array_equal(h5.File(bytes(raw))["d"].read(), arr)


def _scipy_matlab_data():
    scipy_io = pytest.importorskip("scipy.io")
    d = os.path.join(os.path.dirname(scipy_io.matlab.__file__), "tests", "data")
    h5_file = os.path.join(d, "testhdf5_7.4_GLNX86.mat")
    v5_file = os.path.join(d, "testdouble_7.1_GLNX86.mat")
    if not (os.path.exists(h5_file) and os.path.exists(v5_file)):
        pytest.skip("scipy's MATLAB test files are not installed")
    return scipy_io, h5_file, v5_file


def test_reader_on_a_file_the_hdf5_library_wrote():
    """A file written by the HDF5 library itself (MATLAB 7.3 format through
    libhdf5, shipped as test data with scipy): a 512-byte user block, then a
    version 0 superblock with base address 512, the root group as a symbol
    table, a contiguous float64 dataset and a string attribute -- the
    structures of the HDF5 1.6/1.8 output PyTables writes.  The values equal
    those scipy reads from the same variable saved in MATLAB's own format."""
    scipy_io, h5_file, v5_file = _scipy_matlab_data()
    assert h5.is_hdf5(h5_file)
    f = h5.File(h5_file)
    assert f.keys() == ["testdouble"]
    d = f["testdouble"]
    assert d.shape == (9, 1) and d.dtype == np.dtype("<f8")
    assert str(d.attrs["MATLAB_class"]) == "double"
    ref = scipy_io.loadmat(v5_file)["testdouble"]   # MATLAB's 1 x 9, stored column-major
    got = d.read()
    assert np.array_equal(got.T, ref)
    assert np.array_equal(got.ravel(), np.arange(9) * np.pi / 4)
    # absolute addresses in that file are relative to the superblock
    assert f.b.base == 512
