"""bench.py's GB300 arm on a small workload, with the arms that make the
library print (the drainage ladder mirrors the reference's "Step N" and
"t = ... max_abs_err" lines): the result line must be the last line of
stdout and carry value, roofline, cpu_baseline and e2e."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_gb300_arm_line_is_last(gpu):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--n", "64", "--steps", "2", "--warmup", "3",
                        "--cpu-nz", "16", "--cpu-steps", "1", "--e2e-calls", "1", "--no-batched", "--no-adjoint"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [line for line in r.stdout.splitlines() if line.strip()]
    assert lines, r.stderr[-3000:]
    d = json.loads(lines[-1])
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 2
    for key in ("roofline", "cpu_baseline", "e2e", "clocks", "gpu_launches"):
        assert d.get(key) is not None, key
    assert d["gpu_launches"] > 0
    e = d["e2e"]
    assert e["value"] > 0 and e["inner_steps"] >= 1
    assert e["h2d_bytes_per_step"] * e["inner_steps"] == pytest.approx(e["h2d_bytes_per_call"], rel=0.01)
    assert d["ladder_64_eno2"]["files_identical"]
    # the library's progress lines went to stderr, not after the result line
    assert "max_abs_err" in r.stderr
