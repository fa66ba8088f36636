import os
import subprocess
import sys

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def lib():
    """The native library (built in-tree if missing)."""
    from x3dcore2_gb300 import abi, build
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return abi.load()


@pytest.fixture(scope="session")
def oracle():
    import oracle_bind as ob
    if not os.path.exists(ob.ORACLE_LIB):
        ob.build_oracle()
    return ob.oracle()


@pytest.fixture(scope="session")
def reference():
    """The compiled reference: built from the reference checkout, or from the unmodified copy of
    its sources shipped in the reference install folder; skipped where neither exists."""
    import oracle_bind as ob
    if not ob.reference_available():
        if ob.reference_src() is None:
            pytest.skip("reference sources not present on this machine")
        ob.build_reference()
    return ob.reference()


@pytest.fixture(scope="session")
def ctx(lib):
    from x3dcore2_gb300.core import Context
    c = Context(0)
    yield c
    c.close()
