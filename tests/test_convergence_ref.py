"""Simulation.is_converged against the reference's own convergence check.

tests/golden/ref_convergence.json holds the decisions of the reference's
Convergence class (interface/nmag/convergence.py, run unmodified by
tests/golden/make_ref_convergence.py) for seeded sequences of max dm/dt
around the stopping value, with None where no advance has set max dm/dt
yet (main.py:2737-2760).
"""
import json
import os

import nmag

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_convergence.json")


def test_is_converged_matches_reference_decisions():
    g = json.load(open(GOLDEN))
    for case in g["cases"]:
        sim = nmag.Simulation("conv")
        sim.stopping_dm_dt = g["stopping_dm_dt"]
        got = []
        for v in case["max_dm_dt"]:
            sim.max_dm_dt = v
            got.append(bool(sim.is_converged()))
            assert sim.clock.convergence == got[-1]
        assert got == case["converged"]
