"""float_set / vector_set bit for bit against the reference's own sets
module: tests/golden/ref_sets.json holds its results (as float.hex) on
hand-written and seeded random specifications, made by running
interface/nsim/sets.py unmodified (tests/golden/make_ref_sets.py)."""
import json
import os

from nmag import float_set, vector_set

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_sets.json")


def _hex(seq):
    return [float(v).hex() for v in seq]


def test_float_set_matches_reference_module():
    g = json.load(open(GOLDEN))
    for c in g["float_set"]:
        assert _hex(float_set(c["spec"], c["units"])) == c["out"], (c["spec"], c["units"])


def test_vector_set_matches_reference_module():
    g = json.load(open(GOLDEN))
    for c in g["vector_set"]:
        got = vector_set(c["spec"], c["direction"], units=c["units"], normalize=c["normalize"])
        assert [_hex(row) for row in got] == c["out"], (c["spec"], c["direction"], c["normalize"], c["units"])
