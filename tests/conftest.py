"""Shared fixtures: the GB300 library, the CPU oracle and the reference build."""
import os
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lsmpqs-1.0_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
ORACLE_LIBM_LIB = os.path.join(ORACLE_DIR, "liboracle_libm.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libqss_ref.so")
SCRATCH = os.path.join(ROOT, ".test_tmp")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")
    # the tests' scratch files (per-step files, array files, option decks)
    # stay inside the repository: tempfile's directories and pytest's tmp_path
    os.makedirs(SCRATCH, exist_ok=True)
    tempfile.tempdir = SCRATCH
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(SCRATCH, "pytest")


def _ensure_oracle():
    if not os.path.exists(ORACLE_LIB) or not os.path.exists(ORACLE_LIBM_LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so", "liboracle_libm.so"], check=True)


@pytest.fixture(scope="session")
def oracle():
    import qssgpu as Q

    _ensure_oracle()
    lib = Q.load(ORACLE_LIB)
    lib.oracle_set_threads(1)
    return lib


@pytest.fixture(scope="session")
def oracle_libm():
    """The oracle with the platform libm's sin/cos (the reference as linked)
    in place of the portable evaluation both the oracle and the GPU use."""
    import qssgpu as Q

    _ensure_oracle()
    lib = Q.load(ORACLE_LIBM_LIB)
    lib.oracle_set_threads(1)
    return lib


@pytest.fixture(autouse=True)
def _oracle_one_thread(request):
    """The reference's CFL step depends on the OpenMP thread count; other
    libraries in the process (torch) may resize the shared OpenMP pool, so
    every test that uses the oracle starts it on one thread."""
    for name in ("oracle", "oracle_libm"):
        if name in request.fixturenames:
            request.getfixturevalue(name).oracle_set_threads(1)
    yield


@pytest.fixture(scope="session")
def ref():
    import qssgpu as Q

    if not os.path.exists(REF_LIB):
        pytest.skip("reference C build (oracle/_ref) not present on this machine")
    lib = Q.load(REF_LIB)
    lib.oracle_set_threads  # noqa: B018  (the restated kernels export it too)
    return lib


@pytest.fixture(scope="session")
def gpu():
    import qssgpu as Q

    if not os.path.exists(Q.GPU_LIB):
        raise RuntimeError("libqssgpu.so is not built (run __graft_entry__.build())")
    lib = Q.load(Q.GPU_LIB)
    if not lib.qssgpu_device_available():
        raise RuntimeError("the GB300 library sees no CUDA device")
    lib.qssgpu_clear_error()
    lib.qssgpu_set_slabs(1)
    yield lib
    lib.qssgpu_set_slabs(0)
