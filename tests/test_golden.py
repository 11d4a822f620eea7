"""The oracle against golden vectors made by the reference's own C drivers
(compiled unchanged, linked to the restated kernels): drainage, imbibition,
the constant-curvature model, trapping and reinitialisation, with 1-3 OpenMP
threads.  Outputs are compared through SHA-256 of every array (bit for bit)."""
import json
import os

import pytest

import golden_cases as G

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_cases.json")))


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_matches_reference_golden(oracle, name):
    case = G.CASES[name]
    oracle.oracle_set_threads(case.get("threads", 1))
    try:
        rec = G.run_case(oracle, case)
    finally:
        oracle.oracle_set_threads(1)
    want = GOLD[name]
    assert rec["inputs"] == want["inputs"], "seeded inputs differ on this machine"
    assert rec["scalars"] == want["scalars"]
    assert rec["files"] == want["files"]
    bad = [k for k in want["arrays"] if rec["arrays"][k] != want["arrays"][k]]
    assert bad == []
