import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "haskell-abinitio_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"
# The reference checkout, only where REFERENCE_ROOT names it (tests that read
# it skip otherwise and fall back to the committed fixtures).
REFERENCE = Path(os.environ["REFERENCE_ROOT"]) if os.environ.get("REFERENCE_ROOT") else None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


def golden(name):
    return json.loads((GOLDEN / name).read_text())


@pytest.fixture(scope="session")
def ctx():
    """A libgbhf context on cuda:0 (GPU tests only; fails loudly without the library)."""
    import __graft_entry__  # noqa: F401  (path setup)
    from gbhf import build, _lib
    build.build()
    c = _lib.Context(0)
    yield c
    c.close()
