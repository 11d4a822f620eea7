"""bench.py's contract without a GPU: the reference arm (the oracle on the
host cores) prints one JSON line with the keys the contract asks for, as the
last (and only) line of stdout even when C code printed before it, and the
GB300 arm refuses to run on a machine without a CUDA device instead of
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
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 1
    d = json.loads(lines[-1])
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


def test_result_line_is_last_after_buffered_c_output():
    """The library's printf lines (the reference's progress output) sit in
    libc's stdout buffer until exit; the result line must still be the last
    line of stdout, and the C lines must not be lost."""
    code = (
        "import ctypes, sys; sys.path.insert(0, %r); import bench\n"
        "out = bench.ResultLine()\n"
        "libc = ctypes.CDLL(None)\n"
        "libc.printf(b'Step 1: a = 1.250000\\n')\n"
        "print('python progress line')\n"
        "out.emit({'value': 1.0})\n"
        "libc.printf(b'')\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout == json.dumps({"value": 1.0}) + "\n"
    assert "Step 1: a = 1.250000" in r.stderr and "python progress line" in r.stderr
