"""Magnetisation sites of several materials (interface/nmag/nmag_lam.py:
183-330, src/fem.ml:2434-2930).

nmag gives every magnetic material X its own field m_X, defined on the
nodes of the simplices of the regions that carry X ("sites" of X).  A node
on the interface between two materials therefore carries one m per
material; the materials' exchange operators act on their own sites only
(op_H_exch is assembled over X's simplices), so m_A and m_B are not
exchange-coupled across the interface, while the demagnetising potential
lives on the nodes of the whole magnetic mesh and sees the charges of all
materials.

``SiteLayer`` is that bookkeeping, built on the host: per material its
simplices, its sites (mesh nodes, ascending) and the simplices renumbered
to sites, plus the node -> sites map the charge scatter needs.  Sites are
numbered material by material (materials in the order given), which is the
layout of the per-site arrays (m, H_exch, dm/dt, ...) of every material
concatenated.
"""
from __future__ import annotations

import numpy as np


class SiteLayer(object):
    """Sites of the materials of a mesh.

    mesh: an ``nmag.mesh.Mesh`` (regions 1, 2, ...; no vacuum simplices);
    region_materials: for region id r (1-based), ``region_materials[r - 1]``
    lists the names of the materials that region carries (one or several).
    """

    def __init__(self, mesh, region_materials):
        regions = np.asarray(mesh.regions)
        if np.any(regions < 1) or np.any(regions > len(region_materials)):
            raise ValueError("SiteLayer: every simplex needs a region 1..%d" % len(region_materials))
        names = []
        for mats in region_materials:
            for name in mats:
                if name not in names:
                    names.append(name)
        self.materials = names
        self.n_nodes = mesh.n_nodes
        self.tets, self.nodes, self.site_tets, self.offset = [], [], [], []
        off = 0
        for name in names:
            rids = [r + 1 for r, mats in enumerate(region_materials) if name in mats]
            t = np.nonzero(np.isin(regions, rids))[0].astype(np.int64)
            nodes = np.unique(mesh.simplices[t])
            local = np.full(mesh.n_nodes, -1, dtype=np.int64)
            local[nodes] = np.arange(len(nodes))
            self.tets.append(t)
            self.nodes.append(nodes)
            self.site_tets.append(local[mesh.simplices[t]].astype(np.int32))
            self.offset.append(off)
            off += len(nodes)
        self.n_sites = off
        self.site_node = np.concatenate(self.nodes) if names else np.zeros(0, dtype=np.int64)
        self.site_material = np.concatenate([np.full(len(n), k, dtype=np.int32) for k, n in enumerate(self.nodes)]) \
            if names else np.zeros(0, dtype=np.int32)
        # node -> its sites (one per material present there), materials in order
        order = np.argsort(self.site_node, kind="stable")
        counts = np.bincount(self.site_node, minlength=mesh.n_nodes)
        self.node_site_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.node_site_idx = order.astype(np.int64)

    def material_index(self, name):
        return self.materials.index(name)

    def sites_of(self, name):
        """Global site indices of a material's sites."""
        k = self.material_index(name)
        return np.arange(self.offset[k], self.offset[k] + len(self.nodes[k]))

    def site_index(self, name, node):
        """The site of a material at a mesh node; KeyError where the
        material is not defined (as fefields.set_field_at_site fails there)."""
        k = self.material_index(name)
        j = np.searchsorted(self.nodes[k], node)
        if j >= len(self.nodes[k]) or self.nodes[k][j] != node:
            raise KeyError("material %r has no site at node %d" % (name, node))
        return self.offset[k] + int(j)

    def submesh(self, name, points):
        """(points, simplices) of a material's sites: its own mesh, whose
        outer surface is where the material ends (regions of other materials
        and the outside alike)."""
        k = self.material_index(name)
        return np.asarray(points)[self.nodes[k]], self.site_tets[k]

    def scatter(self, per_site):
        """Sum per-site values (S,) or (S, ...) onto the nodes, each node's
        sites in material order."""
        v = np.asarray(per_site)
        out = np.zeros((self.n_nodes,) + v.shape[1:], dtype=v.dtype)
        np.add.at(out, self.site_node, v)   # in site order: a node's sites in material order
        return out

    def gather(self, per_node):
        """Node values at every site."""
        return np.asarray(per_node)[self.site_node]
