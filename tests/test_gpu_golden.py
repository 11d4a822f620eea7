"""The GB300 library against the golden vectors made by the reference's own C
drivers (tests/golden/golden_cases.json), independently of the oracle."""
import json
import os

import pytest

import golden_cases as G
import qssgpu as Q

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_cases.json")))


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_gpu_matches_reference_golden(gpu, name):
    case = G.CASES[name]
    gpu.qssgpu_set_slabs(case.get("threads", 1))
    try:
        rec = G.run_case(gpu, case)
    finally:
        gpu.qssgpu_set_slabs(1)
    Q.check(gpu)
    want = GOLD[name]
    assert rec["inputs"] == want["inputs"], "seeded inputs differ on this machine"
    assert rec["scalars"] == want["scalars"]
    assert rec["files"] == want["files"]
    bad = [k for k in want["arrays"] if rec["arrays"][k] != want["arrays"][k]]
    assert bad == []
