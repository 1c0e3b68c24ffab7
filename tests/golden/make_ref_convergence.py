"""Generate tests/golden/ref_convergence.json: the reference's convergence
decisions, from its own code.

interface/nmag/convergence.py (the Convergence class behind
Simulation.is_converged, main.py:2737-2760) is plain Python that runs
unmodified under Python 3.  Its one import, nsim.circular.CircularList (a
bounded list that only feeds its debugging log and does not parse under
Python 3), is replaced by a list stand-in.  This script drives check(step,
max_dm_dt, stopping_dm_dt, tol_factor) with seeded sequences of max dm/dt
around the stopping value and records, per call, whether it reported
convergence -- what main.py:2751 stores in clock.convergence.  Calls with
max_dm_dt None are not passed to check (main.py:2741 returns False first).

Run (in a tree that has the reference):  python tests/golden/make_ref_convergence.py
"""
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("NMAG_REFERENCE_INTERFACE", "/root/reference/interface")


def load_convergence():
    class CircularList(list):
        def __init__(self, size):
            list.__init__(self)
            self.size = size

        def get_list(self):
            return list(self)

    nsim = types.ModuleType("nsim")
    circ = types.ModuleType("nsim.circular")
    circ.CircularList = CircularList
    nsim.circular = circ
    sys.modules.setdefault("nsim", nsim)
    sys.modules["nsim.circular"] = circ
    spec = importlib.util.spec_from_file_location("ref_convergence", os.path.join(REF, "nmag", "convergence.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def sequences():
    rng = np.random.default_rng(2024)
    out = []
    stop = 1.0
    # hand-made: single dips, pairs, runs of three, None gaps
    out.append([2.0, 0.5, 2.0, 0.5, 0.5, 0.5, 0.5, 0.5, 3.0, 0.9, None, 0.9, 0.8, 1.0, 0.99, 0.99])
    out.append([None, None, 0.1, 0.1, 0.1, 0.1, 0.1])
    for _ in range(6):   # noisy decays across the threshold
        n = 60
        base = np.exp(-np.linspace(0.0, 4.0, n)) * 8.0
        seq = list(base * np.exp(0.6 * rng.standard_normal(n)))
        for k in rng.choice(n, 5, replace=False):
            seq[int(k)] = None
        out.append(seq)
    return stop, out


def main():
    mod = load_convergence()
    stop, seqs = sequences()
    cases = []
    for seq in seqs:
        c = mod.Convergence()
        flags = []
        for step, v in enumerate(seq):
            if v is None:
                flags.append(False)
                continue
            converged, _ = c.check(step, float(v), stop, 1.0)
            flags.append(bool(converged))
        cases.append({"max_dm_dt": [None if v is None else float(v) for v in seq], "converged": flags})
    with open(os.path.join(HERE, "ref_convergence.json"), "w") as f:
        json.dump({"stopping_dm_dt": stop, "cases": cases}, f, indent=0)
    print("wrote", len(cases), "cases")


if __name__ == "__main__":
    main()
