"""nmag's HDF5 data files: ``<name>_dat.h5`` (fields saved by save_data)
and restart files (save_restart_file), in the layout of
nfem/hdf5_v01.py, written and read with nmag.h5:

* /etc/filetype, /etc/fileversion: the tags 'nsimdata', '0.1' (:142-180);
* /mesh: the mesh (:1370-1545; positions in simulation units, /mesh/scale
  with the length of one unit in metres);
* /etc/metadatafields: one row per subfield -- field name, subfield name,
  unit, per-site shape (:771-832);
* /mesh/dofsites: one row holding, per subfield, the sites it lives on
  (first-order sites: one mesh node each; :834-902);
* /data/fields/<field>: one row per save -- id, stage, step, time (s) and
  one column per subfield with its values at its sites in SI (:904-1005);
* /sim, /log: the (empty) groups of save_simulation_files (:287-299).

Restart files carry the clock as the attribute 'clock' of /data/fields/m
(main.py:2764-2857).  Table columns are ordered by name, as PyTables
orders a dictionary-described table.
"""
from __future__ import annotations

import os

import numpy as np

from . import h5
from . import mesh as _mesh

DOFNAME_LEN = 128
UNIT_LEN = 128
MAXIND_LEN = 64
_TABLE = {"CLASS": "TABLE", "VERSION": "2.6"}
_GROUP = {"CLASS": "GROUP", "VERSION": "1.0"}


def _table(rows_by_col, order=None):
    """A structured array from {column: values} with columns by name."""
    names = sorted(rows_by_col) if order is None else order
    cols = [np.asarray(rows_by_col[n]) for n in names]
    dt = np.dtype([(n, c.dtype, c.shape[1:]) for n, c in zip(names, cols)])
    out = np.zeros(len(cols[0]), dt)
    for n, c in zip(names, cols):
        out[n] = c
    return out


def field_rows(meta, rows):
    """The table of one field: rows is a list of dicts with id, stage, step,
    time and {subfield: values} under 'data'; meta: [(subfield, shape)]."""
    cols = {"id": np.array([r["id"] for r in rows], np.int64),
            "stage": np.array([r["stage"] for r in rows], np.int64),
            "step": np.array([r["step"] for r in rows], np.int64),
            "time": np.array([r["time"] for r in rows], np.float64)}
    for name, _ in meta:
        cols[name] = np.stack([np.asarray(r["data"][name], np.float32) for r in rows])
    return _table(cols)


def write(path, msh, metadata, dofsites, tables, sim_units="", clock=None):
    """metadata: [(field, subfield, unit string, shape string)]; dofsites:
    {subfield: int array of node indices}; tables: {field: structured array}."""
    w = h5.Writer()
    w.set_attrs("/", dict(_GROUP, TITLE="", PYTABLES_FORMAT_VERSION="1.6"))
    w.create_group("/etc", dict(_GROUP, TITLE="Configuration and version data"))
    for name, val, title in (("filetype", "nsimdata", "data file type"),
                             ("fileversion", "0.1", "data file type version")):
        w.create_dataset("/etc/" + name, np.array([val.encode("latin-1")]),
                         attrs={"CLASS": "ARRAY", "VERSION": "2.3", "TITLE": title, "FLAVOR": "python"})
    w.create_group("/sim", dict(_GROUP, TITLE="Simulation code and configuration files"))
    w.create_group("/log", dict(_GROUP, TITLE="Log files"))
    w.create_group("/mesh", dict(_GROUP, TITLE="Mesh data"))
    for name, arr in (("points", np.asarray(msh.points, np.float64)), ("simplices", np.asarray(msh.simplices, np.int32)),
                      ("simplicesregions", np.asarray(msh.regions, np.int32))):
        rows = max(1, -(-arr.shape[0] // 64))
        w.create_dataset("/mesh/" + name, arr, chunks=(rows,) + arr.shape[1:], compression=5,
                         attrs={"CLASS": "CARRAY", "VERSION": "1.0", "TITLE": name})
    w.create_group("/mesh/scale", dict(_GROUP, TITLE="Mesh coordinate length scale group"))
    w.create_dataset("/mesh/scale/sifactor", np.float64(1e-9),
                     attrs={"CLASS": "ARRAY", "VERSION": "2.3", "FLAVOR": "python",
                            "TITLE": "Multiply mesh coordinates with this number to obtain meters"})
    meta = _table({"fieldname": np.array([m[0] for m in metadata], "S%d" % DOFNAME_LEN),
                   "dofname": np.array([m[1] for m in metadata], "S%d" % DOFNAME_LEN),
                   "unit": np.array([m[2] for m in metadata], "S%d" % UNIT_LEN),
                   "maxind": np.array([m[3] for m in metadata], "S%d" % MAXIND_LEN)})
    w.create_dataset("/etc/metadatafields", meta,
                     attrs=dict(_TABLE, TITLE="Metadatafields on fields and dofs",
                                simulationunits_str=sim_units, simulationunits_repr=sim_units))
    sites = _table({k: np.asarray(v, np.int32).reshape(1, -1, 1) for k, v in dofsites.items()})
    w.create_dataset("/mesh/dofsites", sites, attrs=dict(_TABLE, TITLE="Sites for all degrees of freedom"))
    w.create_group("/data", dict(_GROUP, TITLE="Simulation data"))
    w.create_group("/data/fields", dict(_GROUP, TITLE="nsim fields"))
    for field, tab in tables.items():
        attrs = dict(_TABLE, TITLE="Field " + field)
        if clock is not None and field == "m":
            attrs["clock"] = clock
        w.create_dataset("/data/fields/" + field, tab, attrs=attrs)
    tmp = path + ".internal"   # written aside and renamed, like main.py:2815-2856
    w.save(tmp)
    os.replace(tmp, path)


def read(path):
    """{'mesh': Mesh, 'metadata': [(field, subfield, unit, shape)],
    'dofsites': {subfield: node indices}, 'tables': {field: structured
    array}, 'clock': the clock attribute of /data/fields/m or None}."""
    f = h5.File(path)
    tag = (_mesh._tag(f, "filetype"), _mesh._tag(f, "fileversion"))
    if tag != ("nsimdata", "0.1"):
        raise IOError("File '%s' is tagged %s, not as nsimdata 0.1" % (path, tag))
    g = f["mesh"]
    msh = _mesh.Mesh(np.asarray(g["points"].read(), np.float64), np.asarray(g["simplices"].read(), np.int32),
                     np.asarray(g["simplicesregions"].read(), np.int32))
    meta = []
    if "metadatafields" in f["etc"]:
        t = f["/etc/metadatafields"].read()
        dec = (lambda x: x.decode("latin-1") if isinstance(x, bytes) else str(x))
        meta = [(dec(r["fieldname"]), dec(r["dofname"]), dec(r["unit"]), dec(r["maxind"])) for r in t]
    dofsites = {}
    if "dofsites" in g:
        t = f["/mesh/dofsites"].read()
        for name in t.dtype.names:
            dofsites[name] = np.asarray(t[name][0]).reshape(-1).astype(np.int64)
    tables, clock = {}, None
    if "data" in f and "fields" in f["data"]:
        for field in f["/data/fields"].keys():
            node = f["/data/fields/" + field]
            tables[field] = node.read()
            if field == "m" and "clock" in node.attrs:
                clock = str(node.attrs["clock"])
    return {"mesh": msh, "metadata": meta, "dofsites": dofsites, "tables": tables, "clock": clock}


def _locate(d, subfieldname, id=None, row=None):
    """The field of a subfield (from the metadata) and the table row: the
    row with that id, else row `row` (0 by default; nfem/hdf5_v01.py:1625-1679)."""
    field = None
    for fieldname, dofname, _, _ in d["metadata"]:
        if dofname == subfieldname:
            field = fieldname
            break
    if field is None or field not in d["tables"]:
        raise KeyError("no subfield '%s' saved in this file" % subfieldname)
    tab = d["tables"][field]
    if id is not None:
        hits = np.nonzero(tab["id"] == id)[0]
        if not len(hits):
            raise KeyError("no row with id %d for field '%s'" % (id, field))
        row = int(hits[0])
    elif row is None:
        row = 0
    return field, tab[row]


def get_subfield_from_h5file(filename, subfieldname, id=None, row=None, unit=None):
    """main.py:2915-2956: a subfield's values (SI) at its sites from a saved
    data file, the row with the given id or the row-th row (0 by default)."""
    if unit:
        raise NotImplementedError("This feature is not implemented yet (unit=*).")
    d = read(filename)
    _, r = _locate(d, subfieldname, id, row)
    return np.array(r[subfieldname], dtype=np.float64)


def get_subfield_sites_from_h5file(filename, subfieldname):
    """main.py:2987-3015: the sites of a subfield as saved (one mesh node each)."""
    d = read(filename)
    if subfieldname not in d["dofsites"]:
        raise KeyError("no subfield '%s' saved in this file" % subfieldname)
    return d["dofsites"][subfieldname].reshape(-1, 1)


def get_subfield_positions_from_h5file(filename, subfieldname):
    """main.py:2958-2985: the positions (m) of a subfield's sites, from the
    file's mesh and its length scale."""
    f = h5.File(filename)
    scale = float(np.asarray(f["/mesh/scale/sifactor"].read()).reshape(-1)[0]) \
        if "scale" in f["mesh"] and "sifactor" in f["/mesh/scale"] else 1.0
    d = read(filename)
    sites = get_subfield_sites_from_h5file(filename, subfieldname).reshape(-1)
    return np.asarray(d["mesh"].points)[sites] * scale
