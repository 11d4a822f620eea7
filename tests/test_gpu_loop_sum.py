"""The parallel loop-order sum (qssgpu_loop_sum, also behind every volume
integral) equals a sequential loop of IEEE additions bit for bit, on
sequences built to defeat it: constant contributions, dense and sparse
packs, exact ties at every scale, binade crossings, subnormals, huge dynamic
range, negative values and non-finite values."""
import ctypes as C
import math

import numpy as np
import pytest

import qssgpu as Q

pytestmark = pytest.mark.gpu


def _seq(x):
    s = 0.0
    for v in x.tolist():
        if v != 0.0:
            s = s + v
    return s


def _cases():
    rng = np.random.default_rng(7)
    dV = 0.04 ** 3
    yield "constant dV", np.full(300_000, dV)
    yield "uniform", rng.random(300_000) * dV
    sparse = np.where(rng.random(400_000) < 0.4, dV, 0.0)
    sparse[rng.random(400_000) < 0.05] = rng.random() * dV
    yield "pack-like", sparse
    yield "ties", rng.choice([1.0, 0.5, 0.25, 2.0 ** -53, 3 * 2.0 ** -54, 2.0 ** -52], 200_000)
    yield "dynamic range", rng.random(200_000) * 10.0 ** rng.integers(-20, 6, 200_000)
    yield "with negatives", rng.random(100_000) - 0.3
    yield "large", 1e16 + rng.random(100_000)
    sub = np.concatenate([np.zeros(5000), 1e-300 * rng.random(50_000), np.full(500, 5e-324)])
    yield "tiny and subnormal", sub
    yield "quantised", 2.0 ** -40 * rng.integers(1, 4, 300_000) + 2.0 ** -93 * rng.integers(0, 4, 300_000)
    inf = rng.random(50_000)
    inf[40_000] = math.inf
    yield "infinity", inf
    yield "empty", np.zeros(0)
    yield "single", np.array([0.1])


@pytest.mark.parametrize("name,x", list(_cases()), ids=[c[0] for c in _cases()])
def test_loop_sum_bit_exact(gpu, name, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = C.c_double(-1.0)
    ptr = x.ctypes.data_as(C.POINTER(C.c_double)) if x.size else C.POINTER(C.c_double)()
    assert gpu.qssgpu_loop_sum(ptr, x.size, C.byref(out)) == 0
    Q.check(gpu)
    want = _seq(x)
    assert np.float64(out.value).tobytes() == np.float64(want).tobytes() or (math.isnan(want) and math.isnan(out.value))
