"""The integer-pipe FP64 arithmetic of the GB300 kernels (csrc/qss_emu.cuh),
compiled for the host, equals the host's IEEE-754 double arithmetic bit for
bit: square root, division, product, sum, difference, power-of-two scaling,
comparisons and maxima on every class of operands, also with a reciprocal seed perturbed
by up to 2 units in the last place (the device's approximate reciprocal is
within 1)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "emu_host_check.cpp")
INC = os.path.join(ROOT, "lsmpqs-1.0_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("emu") / "emu_host_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-I", INC, SRC, "-o", exe],
                   check=True)
    return exe


def _run(exe, cases, seed, jitter):
    r = subprocess.run([exe, str(cases), str(seed), str(jitter)], capture_output=True, text=True)
    rows = {}
    for line in r.stdout.splitlines():
        f = line.split()
        if len(f) >= 3 and f[0] in ("sqrt", "div", "mul", "add", "sub", "scale2", "compare", "max_nonneg",
                                     "neg_abs"):
            rows[f[0]] = (int(f[1]), int(f[2]))
        if f and f[0] == "fallbacks_normal":
            rows["fallbacks"] = tuple(int(x) for x in f[1:])
        if f and f[0] == "sqrt_positive":
            rows["sqrt_positive"] = (int(f[1]), int(f[2]))
    return r.returncode, rows, r.stdout


@pytest.mark.parametrize("seed,jitter", [(1, 0), (2, 1), (3, 2)])
def test_emulated_ops_bit_exact(checker, seed, jitter):
    rc, rows, out = _run(checker, 2_000_000, seed, jitter)
    assert rc == 0, out
    for op in ("sqrt", "div", "mul", "add", "sub", "scale2", "compare", "max_nonneg", "neg_abs"):
        n, bad = rows[op]
        assert n > 1_000_000 and bad == 0, out
    # normal operands take the integer path (no native fallback)
    fam, fdiv, fmul, fadd, _ = rows["fallbacks"]
    assert fam > 50_000 and fdiv == 0 and fmul == 0 and fadd == 0, out
    n_pos, f_sqrt = rows["sqrt_positive"]
    assert n_pos > 100_000 and f_sqrt == 0, out


def test_bad_seed_still_exact(checker):
    """A reciprocal seed far off only sends divisions to the native
    fallback; every result stays exact."""
    rc, rows, out = _run(checker, 500_000, 4, 100_000)
    assert rc == 0, out
    assert rows["div"][1] == 0
    assert rows["fallbacks"][1] > 0
