import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "multic-bubble-cuda_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

# The reference checkout (read-only), if present: REF_ROOT, as in oracle/build.py.
from oracle.build import DEFAULT_REF_ROOT  # noqa: E402

REFERENCE_POST = DEFAULT_REF_ROOT / "post"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def built():
    """Compiles the solver library and the checkers once per session."""
    import __graft_entry__

    __graft_entry__.build()
    return True
