"""Generate tests/golden/cubicmesh/*.nmesh: nmesh text files written by the
reference's own structured mesher.

utils/cubicmesh/cubicmesh.c is a stand-alone C program; oracle/Makefile
(target ref-cubicmesh) compiles it unmodified into oracle/_ref/.  This
script runs it on the cases below, so that the tests can check the nmesh
text reader and the mesher's restatement (nmag.mesh.cubicmesh) where the
reference tree is absent:

* ``box``: 4 x 3 x 2 cells of 1 nm, no regions;
* ``slab_x``: 4 x 2 x 1 cells of 1.25 x 1 x 1, regions split at x = 1.25
  and 3.75 (grid planes: vertices on them take no region);
* ``rod_z``: 2 x 3 x 5 cells of 0.5, regions split at z = 0.5 and 1.5;
* ``offgrid_y``: 3 x 3 x 3 cells of 1, one split at y = 1.7 that cuts
  through cells (those simplices take their last vertex's region).

Run (in a tree that has the reference):  python tests/golden/make_ref_cubicmesh.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = {
    "box": ((4.0, 3.0, 2.0), (4, 3, 2), None),
    "slab_x": ((5.0, 2.0, 1.0), (4, 2, 1), "x:1.25,3.75"),
    "rod_z": ((1.0, 1.5, 2.5), (2, 3, 5), "z:0.5,1.5"),
    "offgrid_y": ((3.0, 3.0, 3.0), (3, 3, 3), "y:1.7"),
}


def main():
    import oracle
    if not oracle.build_ref_cubicmesh():
        raise SystemExit("the reference tree is needed to build its mesher")
    out = os.path.join(HERE, "cubicmesh")
    os.makedirs(out, exist_ok=True)
    for name, (sizes, divisions, flt) in CASES.items():
        path = os.path.join(out, name + ".nmesh")
        oracle.ref_cubicmesh(path, sizes, divisions, flt)
        print("wrote", path)


if __name__ == "__main__":
    main()
