"""Generates the golden fixtures of the level-set path from the reference's own
C drivers (src/level_set_evolution/*.c, src/connectivity/*.c, ... compiled
unchanged by `make -C oracle ref`) linked against the restated 3-D kernels.

    python tests/golden/make_golden.py      # needs oracle/_ref/libqss_ref.so

Each case records the SHA-256 of its seeded inputs and of every output array,
plus the scalar results, in tests/golden/golden_cases.json.  The inputs are
rebuilt from the seeds wherever the tests run, so the fixture stays a few KB.
"""
import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "lsmpqs-1.0_gb300"))
sys.path.insert(0, os.path.dirname(HERE))

import golden_cases as G  # noqa: E402
import qssgpu as Q  # noqa: E402


def main():
    lib = Q.load(os.path.join(ROOT, "oracle", "_ref", "libqss_ref.so"))
    out = {}
    for name, case in G.CASES.items():
        lib.oracle_set_threads(case.get("threads", 1))
        rec = G.run_case(lib, case)
        out[name] = rec
        print(name, rec["scalars"])
    lib.oracle_set_threads(1)
    with open(os.path.join(HERE, "golden_cases.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
