"""Generate tests/golden/ref_sets.json: float_set / vector_set results of
the reference's own sets module.

interface/nsim/sets.py imports only math and runs unmodified under Python
3 (its arithmetic is on floats throughout, so Python 3's division and
rounding give Python 2's results: a half-integer step count fails the
integrality test under either rounding).  This script evaluates it on the
hand-written specifications below and on seeded random ones (both
syntaxes, chained pieces, descending ranges, with and without units) and
stores the results bit for bit (float.hex).

Run (in a tree that has the reference):  python tests/golden/make_ref_sets.py
"""
import importlib.util
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("NMAG_REFERENCE_INTERFACE", "/root/reference/interface")


def load_sets():
    spec = importlib.util.spec_from_file_location("ref_sets", os.path.join(REF, "nsim", "sets.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def specs():
    out = [
        [0, 1, [], 9], [9, 8, [], 0], [0, [9], 9], [0, 0.1, [], 0.45], [0, -0.1, [], -0.45],
        [0, 0.1, [], 0.5, 1, [], 3], [0, [3], 3, 4, [], 6], [1.0, 1.25, "...", 2.0], [0, 2, [], 5],
        [-1, [7], 1], [0.3, 0.7, [], 3.1], [5], [1, 2, 3], [0, 1e-3, [], 0.05],
    ]
    rng = np.random.default_rng(7)
    for _ in range(24):
        pieces = []
        x = float(np.round(rng.uniform(-5, 5), 3))
        pieces.append(x)
        for _ in range(int(rng.integers(1, 4))):
            if rng.random() < 0.5:
                step = float(np.round(rng.uniform(0.05, 1.5), 3)) * (1 if rng.random() < 0.7 else -1)
                n = float(rng.uniform(1.2, 12.0))
                end = float(np.round(x + step * n, 3))
                pieces += [float(np.round(x + step, 6)), [], end]
                x = end
            else:
                n = int(rng.integers(1, 9))
                end = float(np.round(x + rng.uniform(-4, 4), 3))
                pieces += [[n], end]
                x = end
        out.append(pieces)
    return out


def main():
    ref = load_sets()
    hexl = lambda seq: [float(v).hex() for v in seq]
    fl = []
    for s in specs():
        for units in (None, 2.5):
            fl.append({"spec": s, "units": units, "out": hexl(ref.float_set(s, units))})
    vs = []
    for s in specs()[:10]:
        for direction in ([1, 2, 3], [0.3, -1.7, 0.05], [1, 1, 1], [0.7315, 2.2, -0.123]):
            for normalize in (True, False):
                for units in (None, 1e-3):
                    v = ref.vector_set(s, direction, units=units, normalize=normalize)
                    vs.append({"spec": s, "direction": direction, "normalize": normalize, "units": units,
                               "out": [hexl(row) for row in v]})
    with open(os.path.join(HERE, "ref_sets.json"), "w") as f:
        json.dump({"float_set": fl, "vector_set": vs}, f, separators=(",", ":"))
    print("wrote", len(fl), "float_set and", len(vs), "vector_set cases")


if __name__ == "__main__":
    main()
