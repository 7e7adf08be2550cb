import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


try:
    import hypothesis  # noqa: F401
    _HAVE_HYPOTHESIS = True
except ImportError:
    _HAVE_HYPOTHESIS = False

# The oracle's property tests (CPU only) need hypothesis; where it is not
# installed the module is left out of collection, and the header says so.
collect_ignore = [] if _HAVE_HYPOTHESIS else ["test_oracle_properties.py"]


def pytest_report_header(config):
    if not _HAVE_HYPOTHESIS:
        return "hypothesis not installed: tests/test_oracle_properties.py (CPU property tests of the oracle) not collected"
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """The product's C-ABI library, built in-tree if missing."""
    from simplefluid_gb300 import _capi
    if not os.path.exists(_capi.LIB_PATH):
        from simplefluid_gb300 import build
        build.build()
    return _capi.load()


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle as O
    O.build()
    return O

