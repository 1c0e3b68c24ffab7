"""Meshes for the LLG path: a structured box mesher and the nmesh ASCII format.

``box_mesh`` builds the structured grids the benchmark configurations use: a
box of nx*ny*nz cells, each split into the six tetrahedra of the Kuhn
(Freudenthal) subdivision along the cell's main diagonal.  Node order is
x-fastest (node = i + (nx+1)*(j + (ny+1)*k)); tetrahedra are listed cell by
cell (x-fastest) and, within a cell, by the axis permutation of the monotone
path from the cell's (0,0,0) corner to its (1,1,1) corner, in lexicographic
order.  (The reference's own structured mesher, utils/cubicmesh/cubicmesh.c
:60-81,283-345, uses a mirrored split; the configurations here name the Kuhn
split.  ``cubicmesh`` restates that mesher: the same nodes, simplices and
regions as its files.)

``load_ascii``/``save_ascii`` read and write the "# PYFEM mesh file version
1.0" text format (writer: utils/cubicmesh/cubicmesh.c:348-385; reader:
src/mesh.ml:6619-6760 behind interface/nmeshlib/lib1.py:838-863): points,
then "region v0 v1 v2 v3" per simplex, then surfaces, which are skipped, and
periodic point groups, which are refused.
"""
from __future__ import annotations

import itertools
import os
import re

import numpy as np


class Mesh(object):
    """Points (N,3) float64, simplices (T,4) int32, regions (T,) int32."""

    def __init__(self, points, simplices, regions=None):
        self.points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.simplices = np.ascontiguousarray(simplices, dtype=np.int32).reshape(-1, 4)
        if regions is None:
            regions = np.ones(len(self.simplices), dtype=np.int32)
        self.regions = np.ascontiguousarray(regions, dtype=np.int32).reshape(-1)
        if len(self.regions) != len(self.simplices):
            raise ValueError("one region per simplex required")
        if len(self.simplices) and (self.simplices.min() < 0 or self.simplices.max() >= len(self.points)):
            raise ValueError("simplex refers to a point that does not exist")

    @property
    def n_nodes(self):
        return len(self.points)

    @property
    def n_tets(self):
        return len(self.simplices)

    def scaled(self, factor):
        return Mesh(self.points * factor, self.simplices, self.regions)

    def tet_volumes(self):
        """|det| / 6 per simplex."""
        p = self.points[self.simplices]
        return np.abs(np.linalg.det(p[:, 1:] - p[:, :1])) / 6.0

    def locate(self, pos, eps=1e-10):
        """(simplex, barycentric coordinates (4,)) of a point, or None when it
        lies outside every simplex; on a shared face or edge the first
        simplex containing it is taken (P1 fields agree there)."""
        if getattr(self, "_inv", None) is None:
            p = self.points[self.simplices]
            self._p0 = p[:, 0]
            self._inv = np.linalg.inv(np.transpose(p[:, 1:] - p[:, :1], (0, 2, 1)))
        x = np.asarray(pos, dtype=np.float64).reshape(3)
        lam = np.einsum("tij,tj->ti", self._inv, x[None, :] - self._p0)
        bary = np.concatenate([1.0 - lam.sum(1, keepdims=True), lam], axis=1)
        inside = np.nonzero(bary.min(1) >= -eps)[0]
        if len(inside) == 0:
            return None
        t = int(inside[0])
        return t, bary[t]

    def interpolate(self, values, pos, eps=1e-10):
        """Value of the P1 (nodal) field ``values`` (N, ...) at ``pos``, or None
        outside the mesh."""
        hit = self.locate(pos, eps)
        if hit is None:
            return None
        t, bary = hit
        v = np.asarray(values, dtype=np.float64)[self.simplices[t]]
        return np.tensordot(bary, v, axes=(0, 0))


_PERMS = list(itertools.permutations((0, 1, 2)))


def box_mesh(nx, ny, nz, hx, hy=None, hz=None, origin=(0.0, 0.0, 0.0), region=1):
    """Structured Kuhn-split box mesh of nx*ny*nz cells with spacings hx, hy, hz."""
    hy = hx if hy is None else hy
    hz = hx if hz is None else hz
    nx1, ny1, nz1 = nx + 1, ny + 1, nz + 1
    ii, jj, kk = np.meshgrid(np.arange(nx1), np.arange(ny1), np.arange(nz1), indexing="ij")
    pts = np.empty((nz1, ny1, nx1, 3))
    pts[..., 0] = origin[0] + hx * ii.transpose(2, 1, 0)
    pts[..., 1] = origin[1] + hy * jj.transpose(2, 1, 0)
    pts[..., 2] = origin[2] + hz * kk.transpose(2, 1, 0)
    pts = pts.reshape(-1, 3)

    def nid(i, j, k):
        return i + nx1 * (j + ny1 * k)

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci = ci.transpose(2, 1, 0).reshape(-1)
    cj = cj.transpose(2, 1, 0).reshape(-1)
    ck = ck.transpose(2, 1, 0).reshape(-1)
    tets = np.empty((len(ci), 6, 4), dtype=np.int64)
    for p, perm in enumerate(_PERMS):
        off = np.zeros(3, dtype=np.int64)
        tets[:, p, 0] = nid(ci, cj, ck)
        for s, ax in enumerate(perm):
            off[ax] += 1
            tets[:, p, s + 1] = nid(ci + off[0], cj + off[1], ck + off[2])
    tets = tets.reshape(-1, 4).astype(np.int32)
    return Mesh(pts, tets, np.full(len(tets), region, dtype=np.int32))


def cube_mesh(edge_cells=10, h=3.0):
    """The 30 nm cube of the plain-method configuration: 10^3 cells of 3 nm."""
    return box_mesh(edge_cells, edge_cells, edge_cells, h)


def film_mesh():
    """The 500 x 125 x 3 nm film: 200 x 50 x 2 cells of 2.5 x 2.5 x 1.5 nm."""
    return box_mesh(200, 50, 2, 2.5, 2.5, 1.5)


# One cell of the reference's structured mesher split into six tetrahedra,
# each vertex given as its corner offset (x, y, z) in {0, 1}.  Along an axis
# on which the cell's index is odd the offsets are mirrored (1 - c), so that
# neighbouring cells split their shared face along the same diagonal and the
# mesh is conforming.  Split, vertex order and mirroring are the reference's
# (utils/cubicmesh/cubicmesh.c:60-81 for the split, :315-345 for the
# mirroring), so the simplices come out identical to its files.
_CUBICMESH_CELL = np.array([
    [(1, 0, 1), (0, 1, 0), (1, 0, 0), (1, 1, 1)],
    [(1, 0, 1), (0, 1, 0), (0, 1, 1), (0, 0, 0)],
    [(1, 0, 1), (0, 1, 0), (1, 1, 1), (0, 1, 1)],
    [(0, 1, 1), (1, 0, 1), (0, 0, 0), (0, 0, 1)],
    [(1, 0, 1), (0, 1, 0), (0, 0, 0), (1, 0, 0)],
    [(1, 0, 0), (0, 1, 0), (1, 1, 0), (1, 1, 1)],
], dtype=np.int64)


def _cubicmesh_filter(spec):
    """(axis, thresholds) of the mesher's region filter: "x:1.5,3.0" (axis
    x, y, z or its number, then ascending coordinates; cubicmesh.c:167-203)."""
    if isinstance(spec, str):
        head, _, rest = spec.partition(":")
        axis = {"x": 0, "y": 1, "z": 2}.get(head.strip())
        if axis is None:
            try:
                axis = int(head)
            except ValueError:
                raise ValueError("region filter '%s': give the axis as x, y, z or 0-2, then ':'" % spec)
        thresholds = [float(v) for v in rest.split(",") if v.strip()] if rest else []
    else:
        axis, thresholds = int(spec[0]), [float(v) for v in spec[1]]
    if axis not in (0, 1, 2):
        raise ValueError("region filter: axis %r is not one of 0, 1, 2" % (axis,))
    if any(b < a for a, b in zip(thresholds, thresholds[1:])):
        raise ValueError("region filter: the coordinates must be ordered from smaller to greater")
    return axis, thresholds


def _cubicmesh_regions(points, simplices, region_filter):
    """Region of each simplex under the mesher's filter (cubicmesh.c:205-246):
    a vertex beyond the k-th threshold (of k = 0, 1, ... ascending, the
    largest tested first) lies in region k + 2, below all of them in region
    1, and within 1e-10 of a threshold in none; a simplex takes the region of
    its last vertex that has one (-1 when none has)."""
    if region_filter is None:
        return np.ones(len(simplices), dtype=np.int32)
    axis, thr = _cubicmesh_filter(region_filter)
    x = points[:, axis]
    vreg = np.ones(len(points), dtype=np.int64)
    decided = np.zeros(len(points), dtype=bool)
    for k in range(len(thr) - 1, -1, -1):
        d = thr[k] - x
        on = ~decided & (np.abs(d) <= 1e-10)
        vreg[on] = -1
        decided |= on
        beyond = ~decided & (d < 0.0)
        vreg[beyond] = k + 2
        decided |= beyond
    reg = np.full(len(simplices), -1, dtype=np.int64)
    for c in range(simplices.shape[1]):
        r = vreg[simplices[:, c]]
        reg = np.where(r >= 0, r, reg)
    return reg.astype(np.int32)


def cubicmesh(sizes, divisions, region_filter=None):
    """The mesh the reference's structured mesher writes for
    ``cubicmesh out.nmesh,lx:nx,ly:ny,lz:nz [filter]`` (utils/cubicmesh/
    cubicmesh.c:266-345): (nx+1)(ny+1)(nz+1) nodes at (i lx/nx, j ly/ny,
    k lz/nz), numbered with k fastest, then j, then i; six tetrahedra per cell
    (``_CUBICMESH_CELL``), cells in the same order.  Regions are 1, or set by
    ``region_filter`` ("x:1.5,3.0" or (axis, [coordinates]), see
    ``_cubicmesh_regions``).  Coordinates are kept at full precision; the
    mesher's text file rounds them to six decimals."""
    sizes = [float(v) for v in sizes]
    nn = [int(v) for v in divisions]
    if len(sizes) != 3 or len(nn) != 3:
        raise ValueError("cubicmesh: three sizes and three divisions")
    if min(nn) < 1:
        raise ValueError("cubicmesh: the number of cells along each side must be positive")
    if min(sizes) <= 0.0:
        raise ValueError("cubicmesh: the sides must have positive lengths")
    dd = [sizes[a] / nn[a] for a in range(3)]
    ipos = np.stack(np.meshgrid(np.arange(nn[0] + 1), np.arange(nn[1] + 1), np.arange(nn[2] + 1),
                                indexing="ij"), axis=-1).reshape(-1, 3)
    points = np.empty(ipos.shape, dtype=np.float64)
    for a in range(3):
        points[:, a] = ipos[:, a].astype(np.float64) * dd[a]
    cells = np.stack(np.meshgrid(np.arange(nn[0]), np.arange(nn[1]), np.arange(nn[2]), indexing="ij"),
                     axis=-1).reshape(-1, 3)
    odd = (cells % 2 == 1)[:, None, None, :]
    corner = np.where(odd, 1 - _CUBICMESH_CELL[None], _CUBICMESH_CELL[None]) + cells[:, None, None, :]
    node = (corner[..., 0] * (nn[1] + 1) + corner[..., 1]) * (nn[2] + 1) + corner[..., 2]
    simplices = node.reshape(-1, 4).astype(np.int32)
    return Mesh(points, simplices, _cubicmesh_regions(points, simplices, region_filter))


def save_ascii(mesh, filename):
    with open(filename, "w") as f:
        f.write("# PYFEM mesh file version 1.0\n")
        f.write("# dim = 3 \tnodes = %d \tsimplices = %d \tsurfaces = 0 \tperiodic = 0\n"
                % (mesh.n_nodes, mesh.n_tets))
        f.write("%d\n" % mesh.n_nodes)
        for p in mesh.points:
            f.write(" %r %r %r\n" % (float(p[0]), float(p[1]), float(p[2])))
        f.write("%d\n" % mesh.n_tets)
        for r, s in zip(mesh.regions, mesh.simplices):
            f.write(" %d %d %d %d %d\n" % (r, s[0], s[1], s[2], s[3]))
        f.write("0\n0\n")


def magnetic_part(mesh):
    """The simplices of the magnetic regions (region id >= 1; region 0 is
    vacuum, main.py:1190,1297) and the nodes they use, renumbered in their
    original order.  Returns (Mesh, node_map): node k of the result is
    mesh.points[node_map[k]]."""
    keep = mesh.regions >= 1
    simp = mesh.simplices[keep]
    used = np.unique(simp.reshape(-1))
    renum = np.full(mesh.n_nodes, -1, dtype=np.int64)
    renum[used] = np.arange(len(used))
    return Mesh(mesh.points[used], renum[simp].astype(np.int32), mesh.regions[keep]), used


_NMESH_TAG = re.compile(r"# PYFEM mesh file version ([0-9]+)\.([0-9]+)")
_NMESH_SUMMARY = re.compile(r"# dim[ \t]*=[ \t]*([0-9]+)[ \t]*nodes[ \t]*=[ \t]*([0-9]+)[ \t]*"
                            r"simplices[ \t]*=[ \t]*([0-9]+)[ \t]*surfaces[ \t]*=[ \t]*([0-9]+)[ \t]*"
                            r"periodic[ \t]*=[ \t]*([0-9]+)")


def load_ascii(filename):
    """Read an nmesh text file as the reference's reader does (src/mesh.ml
    :6619-6760, read_mesh): line 1 "# PYFEM mesh file version 1.x", line 2
    the summary "# dim = 3 nodes = N simplices = S surfaces = F periodic =
    P" whose counts place the sections (points from line 4, simplices
    "region v0 v1 v2 v3" from line N + 5, then the surfaces, which are
    skipped, and the periodic point groups).  Refused as the reference
    refuses them, with the line number: another major version, a missing
    summary, rows with the wrong number of entries, vertex indices out of
    range or repeated in a simplex.  Periodic point groups (P > 0) are
    refused too: the LLG path here has no periodic identification."""
    if not os.path.exists(filename):
        raise IOError("file '%s' does not exist" % filename)
    with open(filename) as f:
        lines = f.read().splitlines()
    if len(lines) < 2:
        raise IOError("%s: mesh information not specified" % filename)
    tag = _NMESH_TAG.match(lines[0])
    if tag is None:
        raise IOError("%s: version of the file not given (expected '# PYFEM mesh file version 1.0')" % filename)
    if tag.group(1) != "1":
        raise IOError("%s: wrong version of the file (%s.%s)" % (filename, tag.group(1), tag.group(2)))
    summary = _NMESH_SUMMARY.match(lines[1])
    if summary is None:
        raise IOError("%s: mesh summary not given (line 2)" % filename)
    dim, n, t, nsurf, nper = (int(v) for v in summary.groups())
    if dim != 3:
        raise IOError("%s: a %d-dimensional mesh (the LLG path needs 3 dimensions)" % (filename, dim))

    def fields(k, what):
        if k >= len(lines):
            raise IOError("%s - LINE %d: the file ends before the %s" % (filename, k + 1, what))
        return lines[k].split()

    def fail(k, msg):
        raise IOError("%s - LINE %d: %s" % (filename, k + 1, msg))

    pts = np.empty((n, 3), dtype=np.float64)
    for i in range(n):
        k = 3 + i
        row = fields(k, "points")
        if len(row) != dim:
            fail(k, "Wrong number of point coordinates")
        try:
            pts[i] = [float(v) for v in row]
        except ValueError:
            fail(k, "Wrong point coordinates")
    simp = np.empty((t, 4), dtype=np.int32)
    regions = np.empty(t, dtype=np.int32)
    for i in range(t):
        k = 4 + n + i
        row = fields(k, "simplices")
        if len(row) != dim + 2:
            fail(k, "Wrong number of simplex coordinates")
        try:
            idx = [int(v) for v in row[1:]]
        except ValueError:
            fail(k, "Wrong simplex indices")
        bad = [j for j, v in enumerate(idx) if v >= n or v < 0]
        if bad:
            fail(k, "Index %d out of range" % (bad[0] + 1))
        if len(set(idx)) != len(idx):
            fail(k, "Duplicate index")
        try:
            regions[i] = int(row[0])
        except ValueError:
            fail(k, "Wrong number of simplex region")
        simp[i] = idx
    if nper > 0:
        raise IOError("%s: %d periodic point groups: periodic meshes are not supported by this path"
                      % (filename, nper))
    return Mesh(pts, simp, regions)


def _tag(f, name):
    """The first entry of /etc/<name> (a one-element string array), or None."""
    if "etc" not in f or name not in f["etc"]:
        return None
    v = np.asarray(f["/etc/" + name].read()).reshape(-1)
    return v[0].decode("latin-1") if isinstance(v[0], bytes) else str(v[0])


def load_hdf5(filename):
    """Read an nmesh HDF5 file (nmeshlib/lib1.py:773-836): /mesh/points,
    /mesh/simplices, /mesh/simplicesregions, tagged in /etc as an nmesh 1.0
    (or nsimdata 0.1) file.  Periodic point indices are not read (periodic
    boundaries are not part of this path)."""
    from . import h5
    if not os.path.exists(filename):
        raise IOError("file '%s' does not exist" % filename)
    f = h5.File(filename)
    if "mesh" not in f:
        raise IOError("File '%s' does not contain a mesh" % filename)
    if "etc" not in f:
        raise IOError("File '%s' has no /etc node: cannot be nmesh file" % filename)
    tag = (_tag(f, "filetype"), _tag(f, "fileversion"))
    if tag not in (("nmesh", "1.0"), ("nsimdata", "0.1")):
        raise IOError("File '%s' is tagged %s, not as an nmesh 1.0 file" % (filename, tag))
    g = f["mesh"]
    if not all(k in g for k in ("points", "simplices", "simplicesregions")):
        raise IOError("File '%s' is not a valid mesh file: some mesh attributes are missing" % filename)
    pts = np.asarray(g["points"].read(), dtype=np.float64).reshape(-1, 3)
    simp = np.asarray(g["simplices"].read(), dtype=np.int32).reshape(-1, 4)
    reg = np.asarray(g["simplicesregions"].read(), dtype=np.int32).reshape(-1)
    m = Mesh(pts, simp, reg)
    if "scale" in g and "sifactor" in g["scale"]:
        m.sifactor = float(np.asarray(g["/mesh/scale/sifactor"].read()).reshape(-1)[0])
    return m


def save_hdf5(mesh, filename, sifactor=None, unit=None):
    """Write the mesh in the layout of nfem/hdf5_v01.py:1370-1545 (tag
    nmesh 1.0 in /etc; /mesh/points, /mesh/simplices and
    /mesh/simplicesregions as deflate-compressed chunked arrays with
    PyTables' node attributes; the optional /mesh/scale group)."""
    from . import h5
    w = h5.Writer()
    w.set_attrs("/", {"CLASS": "GROUP", "VERSION": "1.0", "TITLE": "", "PYTABLES_FORMAT_VERSION": "1.6"})
    w.create_group("/etc", {"CLASS": "GROUP", "VERSION": "1.0", "TITLE": "Configuration and version data"})
    for name, val, title in (("filetype", "nmesh", "data file type"), ("fileversion", "1.0", "data file type version")):
        w.create_dataset("/etc/" + name, np.array([val.encode("latin-1")]),
                         attrs={"CLASS": "ARRAY", "VERSION": "2.3", "TITLE": title, "FLAVOR": "python"})
    w.create_group("/mesh", {"CLASS": "GROUP", "VERSION": "1.0", "TITLE": "Mesh data"})
    for name, arr, title in (
            ("points", np.asarray(mesh.points, dtype=np.float64), "Positions of mesh nodes (=points)"),
            ("simplices", np.asarray(mesh.simplices, dtype=np.int32),
             "Indices of nodes (starting from zero). Each row is one simplex."),
            ("simplicesregions", np.asarray(mesh.regions, dtype=np.int32), "Region ids (one for each simplex).")):
        rows = max(1, -(-arr.shape[0] // 64))   # at most 64 chunks
        w.create_dataset("/mesh/" + name, arr, chunks=(rows,) + arr.shape[1:], compression=5,
                         attrs={"CLASS": "CARRAY", "VERSION": "1.0", "TITLE": title})
    if sifactor is not None:
        w.create_group("/mesh/scale", {"CLASS": "GROUP", "VERSION": "1.0",
                                       "TITLE": "Mesh coordinate length scale group"})
        w.create_dataset("/mesh/scale/sifactor", np.float64(sifactor),
                         attrs={"CLASS": "ARRAY", "VERSION": "2.3", "FLAVOR": "python",
                                "TITLE": "Multiply mesh coordinates with this number to obtain meters"})
        if unit is not None:
            w.create_dataset("/mesh/scale/unit", np.array(str(unit).encode("latin-1")),
                             attrs={"CLASS": "ARRAY", "VERSION": "2.3", "FLAVOR": "python",
                                    "TITLE": "SI object for coordinate to position conversion"})
    w.save(filename)


def load(filename_or_mesh):
    """A Mesh, or a file in nmesh ASCII (first line "# PYFEM ...") or nmesh
    HDF5 (the HDF5 signature); anything else is refused
    (nmeshlib/lib1.py:656-678,838-863)."""
    if isinstance(filename_or_mesh, Mesh):
        return filename_or_mesh
    from . import h5
    if not os.path.exists(filename_or_mesh):
        raise IOError("file '%s' does not exist" % filename_or_mesh)
    with open(filename_or_mesh, "rb") as f:
        ascii_tag = f.read(7) == b"# PYFEM"
    if ascii_tag:
        return load_ascii(filename_or_mesh)
    if h5.is_hdf5(filename_or_mesh):
        return load_hdf5(filename_or_mesh)
    raise IOError("%s is unknown file format (not ascii, not hdf5)" % filename_or_mesh)
