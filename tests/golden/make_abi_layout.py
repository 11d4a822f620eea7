"""Records sizeof/offsetof of Grid, QSS_DataArrays and Options as laid out by
the reference headers (src/geometry/qss_grid.h, src/utilities/qss_data_arrays.h,
src/utilities/qss_options.h, FP64 build) into tests/golden/abi_layout.json.

    LSMPQS_REF=/path/to/reference python tests/golden/make_abi_layout.py
    python tests/golden/make_abi_layout.py /path/to/reference
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "lsmpqs-1.0_gb300"))
from abi_probe import probe_source  # noqa: E402


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LSMPQS_REF")
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        sys.exit("make_abi_layout: give the reference tree as the argument or in LSMPQS_REF")
    inc = ["-I" + os.path.join(ref, d) for d in ("config", "src/geometry", "src/utilities")]
    hdr = '#include "QSSLIB_config.h"\n#include "qss_grid.h"\n#include "qss_data_arrays.h"\n#include "qss_options.h"\n'
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "p.c")
        with open(src, "w") as f:
            f.write(probe_source(hdr))
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-DQSSLIB_REAL=double", "-DLSMLIB_REAL=double", *inc, src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    layout = json.loads(out)
    with open(os.path.join(HERE, "abi_layout.json"), "w") as f:
        json.dump(layout, f, indent=1, sort_keys=True)
    print(len(layout), "entries")


if __name__ == "__main__":
    main()
