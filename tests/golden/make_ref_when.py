"""Generate tests/golden/ref_when.json: match_time / next_time answers of
the reference's own schedule module.

interface/nsim/when.py runs under Python 3 as imported: its module body
(everything before the ``if __name__ == "__main__":`` demonstration block,
which an import does not execute and which holds its only Python 2 print
statements) is executed unmodified.  Its next_time(tols=...) calls the
Python 2 dict method has_key, so the tolerances are passed as a dict that
has one.  Clocks carry plain numbers (simulation units for the times).
This script evaluates schedules built from at / every / | / & / never on
seeded clock states and stores every answer.

Run (in a tree that has the reference):  python tests/golden/make_ref_when.py
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("NMAG_REFERENCE_INTERFACE", "/root/reference/interface")

IDS = ["step", "stage_step", "stage", "time", "stage_time"]

# schedules as nested lists: ["every", id, delta, first, last], ["at", id, value],
# ["or", a, b], ["and", a, b], ["never"]
SPECS = [
    ["every", "step", 5, 0, None],
    ["every", "step", 3, 2, 22],
    ["every", "stage_step", 10, 0, None],
    ["every", "time", 0.7, 0, None],
    ["every", "stage_time", 2.5, 1.0, 20.0],
    ["every", "stage", 2, 1, None],
    ["at", "step", 15],
    ["at", "time", 3.5],
    ["at", "convergence", True],
    ["at", "stage_end", True],
    ["never"],
    ["or", ["every", "step", 10, 0, None], ["at", "convergence", True]],
    ["or", ["every", "time", 1.5, 0, None], ["every", "time", 4.0, 0, None]],
    ["or", ["every", "stage_step", 4, 0, None], ["every", "time", 2.0, 0, None]],
    ["and", ["every", "step", 2, 0, None], ["every", "step", 3, 0, None]],
    ["and", ["every", "stage", 2, 0, None], ["at", "convergence", True]],
    ["and", ["every", "step", 4, 0, 30], ["every", "stage", 1, 2, None]],
    ["or", ["and", ["every", "step", 2, 0, 21], ["every", "step", 4, 10, None]], ["at", "step", 15]],
    ["or", ["never"], ["every", "step", 7, 0, None]],
]


def load_when():
    src = open(os.path.join(REF, "nsim", "when.py")).read()
    body = src[:src.index('if __name__ == "__main__":')]
    ns = {"__name__": "ref_when"}
    exec(compile(body, os.path.join(REF, "nsim", "when.py"), "exec"), ns)
    return ns


class Tols(dict):
    def has_key(self, k):
        return k in self


def build(ns, spec):
    kind = spec[0]
    if kind == "every":
        return ns["every"](spec[1], spec[2], first=spec[3], last=spec[4])
    if kind == "at":
        return ns["at"](spec[1], spec[2])
    if kind == "never":
        return ns["never"]
    a, b = build(ns, spec[1]), build(ns, spec[2])
    return (a | b) if kind == "or" else (a & b)


def clocks():
    rng = np.random.default_rng(11)
    out = []
    for k in range(30):
        step = int(rng.integers(0, 40))
        out.append({"step": step, "stage_step": int(rng.integers(0, step + 1)), "stage": int(rng.integers(1, 5)),
                    "time": float(np.round(rng.uniform(0, 25), 2)) if k % 3 else 0.7 * int(rng.integers(0, 30)),
                    "stage_time": float(np.round(rng.uniform(0, 22), 2)) if k % 4 else 2.5 * int(rng.integers(0, 9)) + 1.0,
                    "convergence": bool(rng.random() < 0.3), "stage_end": bool(rng.random() < 0.3)})
    return out


def main():
    ns = load_when()
    tols = Tols(time=1e-9, stage_time=1e-9)
    cases = []
    for spec in SPECS:
        w = build(ns, spec)
        res = []
        for c in clocks():
            r = {"match": bool(w.match_time(dict(c))), "next": {}, "next_tol": {}}
            for i in IDS:
                r["next"][i] = w.next_time(i, dict(c))
                r["next_tol"][i] = w.next_time(i, dict(c), tols)
            res.append(r)
        cases.append({"spec": spec, "results": res})
    with open(os.path.join(HERE, "ref_when.json"), "w") as f:
        json.dump({"clocks": clocks(), "tols": dict(tols), "cases": cases}, f, separators=(",", ":"))
    print("wrote", len(cases), "schedules x", len(clocks()), "clocks")


if __name__ == "__main__":
    main()
