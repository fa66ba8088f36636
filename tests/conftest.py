import os
import subprocess
import sys

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

REFERENCE_SRC = "/root/reference/corelib/src"


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
    """The compiled reference (only where its sources exist; never on the GPU host)."""
    import oracle_bind as ob
    if not ob.reference_available():
        if not os.path.isdir(REFERENCE_SRC):
            pytest.skip("reference sources not present on this machine")
        subprocess.run(["make", "-s", "-C", ob.ORACLE_DIR, "ref"], check=True)
    return ob.reference()


@pytest.fixture(scope="session")
def ctx(lib):
    from x3dcore2_gb300.core import Context
    c = Context(0)
    yield c
    c.close()
