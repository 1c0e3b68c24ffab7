"""Meshes for the LLG path: a structured box mesher and the nmesh ASCII format.

``box_mesh`` builds the structured grids the benchmark configurations use: a
box of nx*ny*nz cells, each split into the six tetrahedra of the Kuhn
(Freudenthal) subdivision along the cell's main diagonal.  Node order is
x-fastest (node = i + (nx+1)*(j + (ny+1)*k)); tetrahedra are listed cell by
cell (x-fastest) and, within a cell, by the axis permutation of the monotone
path from the cell's (0,0,0) corner to its (1,1,1) corner, in lexicographic
order.  (The reference's own structured mesher, utils/cubicmesh/cubicmesh.c
:60-81,283-345, uses a mirrored split; the configurations here name the Kuhn
split.)

``load_ascii``/``save_ascii`` read and write the "# PYFEM mesh file version
1.0" text format (writer: utils/cubicmesh/cubicmesh.c:348-385; reader:
interface/nmeshlib/lib1.py:805-863): points, then "region v0 v1 v2 v3" per
simplex, then surfaces and periodic blocks, which are skipped.
"""
from __future__ import annotations

import itertools
import os

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


def load_ascii(filename):
    """Read an nmesh ASCII file (points, region+simplices; surfaces ignored)."""
    if not os.path.exists(filename):
        raise IOError("file '%s' does not exist" % filename)
    with open(filename) as f:
        lines = [ln for ln in (l.strip() for l in f) if ln and not ln.startswith("#")]
    it = iter(lines)
    n = int(next(it).split()[0])
    pts = np.array([[float(v) for v in next(it).split()[:3]] for _ in range(n)], dtype=np.float64)
    t = int(next(it).split()[0])
    rows = [next(it).split() for _ in range(t)]
    regions = np.array([int(r[0]) for r in rows], dtype=np.int32)
    simp = np.array([[int(v) for v in r[1:5]] for r in rows], dtype=np.int32)
    return Mesh(pts, simp, regions)


def load(filename_or_mesh):
    if isinstance(filename_or_mesh, Mesh):
        return filename_or_mesh
    return load_ascii(filename_or_mesh)
