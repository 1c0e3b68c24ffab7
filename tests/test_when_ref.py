"""The save / do schedules against the reference's own when module:
tests/golden/ref_when.json holds match_time / next_time answers (with and
without tolerances) of interface/nsim/when.py, executed as imported by
tests/golden/make_ref_when.py, for schedules built from at / every / | /
& / never on seeded clock states."""
import json
import os

from nmag.when import at, every, never

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_when.json")


def build(spec):
    kind = spec[0]
    if kind == "every":
        return every(spec[1], spec[2], first=spec[3], last=spec[4])
    if kind == "at":
        return at(spec[1], spec[2])
    if kind == "never":
        return never
    a, b = build(spec[1]), build(spec[2])
    return (a | b) if kind == "or" else (a & b)


def same(got, want):
    # the answer's kind matters: True/False (bool) against a next value (number)
    if isinstance(want, bool) or isinstance(got, bool):
        return isinstance(got, bool) and isinstance(want, bool) and got == want
    return got == want


def test_schedules_match_reference_module():
    g = json.load(open(GOLDEN))
    for case in g["cases"]:
        w = build(case["spec"])
        for clock, r in zip(g["clocks"], case["results"]):
            assert w.match_time(dict(clock)) == r["match"], (case["spec"], clock)
            for ident, want in r["next"].items():
                got = w.next_time(ident, dict(clock))
                assert same(got, want), (case["spec"], clock, ident, got, want)
            for ident, want in r["next_tol"].items():
                got = w.next_time(ident, dict(clock), g["tols"])
                assert same(got, want), ("tols", case["spec"], clock, ident, got, want)
