import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcmpy_ed.so")


@pytest.fixture(scope="session")
def golden():
    """Golden vectors produced by the unmodified reference (tests/golden/make_golden.py)."""
    out = {}
    for f in GOLDEN.glob("*.npz"):
        with np.load(f, allow_pickle=False) as d:
            out[f.stem] = {k: d[k] for k in d.files}
    return out


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("this test needs a CUDA GPU")
    from cmpy_gb300 import _native

    _native.lib()
    return torch.device("cuda", 0)
