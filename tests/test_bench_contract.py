"""bench.py's contract without a GPU: the reference arm (the oracle on the
host cores) prints one JSON line with the keys the contract asks for, and
the GB300 arm refuses to run on a machine without a CUDA device instead of
falling back to the CPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args, timeout=300):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_line():
    r = _bench("--impl", "reference", "--n", "48", "--cpu-nz", "8", "--steps", "1", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [line for line in r.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_gpu_arm_fails_without_a_device():
    import qssgpu as Q

    if Q.load(Q.GPU_LIB).qssgpu_device_available():
        import pytest

        pytest.skip("a GPU is present")
    r = _bench("--n", "48", "--steps", "1", "--warmup", "3", "--no-cpu", "--no-batched", "--no-adjoint",
               "--no-ladder", "--no-e2e", timeout=120)
    assert r.returncode != 0
    assert "no CUDA device" in r.stderr
    assert not [line for line in r.stdout.splitlines() if line.startswith("{")]
