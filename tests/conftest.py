import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the reference package checked out beside this repository (or where
# CUSNA_REFERENCE_DIR says); tests that read it skip where it is absent
REFERENCE = os.environ.get("CUSNA_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))
FIXTURES = os.path.join(REFERENCE, "tests", "testthat", "fixtures")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libcusna_gb300.so")


@pytest.fixture(scope="session")
def port():
    """The CPU oracle (C restatement of the reference engine)."""
    import oracle
    oracle.build(ref=False)
    return oracle.Oracle("port")


@pytest.fixture(scope="session")
def ref_engine():
    """The reference engine compiled from its own sources (only where present)."""
    import oracle
    if not os.path.exists(os.path.join(REFERENCE, "src", "libcusna_saom_cpu.cpp")):
        pytest.skip("reference sources not present")
    oracle.build(ref=True)
    return oracle.Oracle("reference")


@pytest.fixture(scope="session")
def fixtures_dir():
    if not os.path.isdir(FIXTURES):
        pytest.skip("reference fixtures not present")
    return FIXTURES


@pytest.fixture(scope="session")
def gpu_lib():
    """libcusna_gb300.so, built in-tree; fails loudly if it cannot load."""
    from cusna_gb300 import build as B
    from cusna_gb300.abi import load_library
    B.build()
    lib = load_library()
    assert lib.cusna_has_cuda() == 1, "no CUDA device visible to libcusna_gb300"
    return lib


@pytest.fixture(scope="session")
def built_lib():
    """libcusna_gb300.so loaded without requiring a device (symbol checks)."""
    from cusna_gb300 import build as B
    from cusna_gb300.abi import load_library
    B.build()
    return load_library()
