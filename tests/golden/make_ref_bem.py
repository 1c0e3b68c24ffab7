"""Generate tests/golden/ref_bem.npz: BEM matrices filled by the reference's
own code.

The reference's Lindholm stub (src/bem3d_stubs.c:413-610) is plain C behind
OCaml value macros.  oracle/Makefile compiles it unmodified against the
project's minimal caml shim (oracle/caml_shim), and oracle/ref_bem_harness.c
drives it the way the reference's row fill does (src/bem3d.ml:938-1047).  This
script runs that fill on three meshes and stores what the tests need where
the reference tree is absent (the GPU machine):

* ``box`` (4 x 3 x 2 cells of 2.0 x 2.5 x 1.5 nm): the whole matrix;
* ``cube`` (the 30 nm cube, 10^3 cells) and ``plate`` (20 x 6 x 2 cells of
  2.5 x 2.5 x 1.5 nm, the film's cell shape): every 43rd (cube) / 29th
  (plate) row, plus the row sums and column sums of the whole matrix.

The surface triangles, normals and solid angles handed to the stub come from
the oracle (its restatement of bem3d.ml:32-181 and mesh.ml:1792-1821).

Run (in a tree that has the reference):  python tests/golden/make_ref_bem.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "nmag-src_gb300"))

MESHES = {
    "box": ((4, 3, 2, 2.0, 2.5, 1.5), None),
    "cube": ((10, 10, 10, 3.0, 3.0, 3.0), 43),
    "plate": ((20, 6, 2, 2.5, 2.5, 1.5), 29),
}


def main():
    import oracle
    from nmag import mesh
    if not oracle.build_ref():
        raise SystemExit("the reference tree is needed (oracle.REF_SRC)")
    out = {}
    for name, (args, every) in MESHES.items():
        msh = mesh.box_mesh(*args)
        om = oracle.OracleMesh(msh.points, msh.simplices)
        R = oracle.ref_bem(om)
        out[name + "_args"] = np.array(args, dtype=np.float64)
        if every is None:
            out[name + "_rows"] = np.arange(om.nb, dtype=np.int32)
            out[name + "_bem"] = R
        else:
            rows = np.arange(0, om.nb, every, dtype=np.int32)
            out[name + "_rows"] = rows
            out[name + "_bem"] = R[rows]
        out[name + "_rowsum"] = R.sum(axis=1)
        out[name + "_colsum"] = R.sum(axis=0)
        print(name, "nb", om.nb, "triangles", om.ntri, "rows kept", len(out[name + "_rows"]))
    np.savez_compressed(os.path.join(HERE, "ref_bem.npz"), **out)


if __name__ == "__main__":
    main()
