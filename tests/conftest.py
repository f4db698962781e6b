import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    """All committed golden vectors (made by tests/golden/make_golden.py from
    the reference's own code), merged into one dict."""
    out = {}
    for f in sorted(GOLDEN.glob("*.npz")):
        with np.load(f, allow_pickle=False) as z:
            out.update({k: z[k] for k in z.files})
    return out
