import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def built():
    """Builds the oracle (and the extension when nvcc is present) once per session."""
    import oracle as orc

    orc.build()
    from morphogenesis_gb300 import build as b

    b.build()
    return True
