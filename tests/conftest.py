import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


@pytest.fixture(scope="session")
def lib():
    """The product library, built in-tree if missing."""
    from simplemoc_gb300 import _lib as L
    if not L.LIB_PATH.exists():
        from simplemoc_gb300 import build
        build.build()
    return L._lib()


@pytest.fixture(scope="session")
def port():
    import oracle
    if not oracle.PORT_LIB.exists():
        oracle.build(reference=False)
    return oracle.Port()


@pytest.fixture(scope="session")
def ref():
    import oracle
    if not oracle.Reference.available():
        if oracle.ref_src() is not None:
            oracle.build(reference=True)
    if not oracle.Reference.available():
        pytest.skip("reference objects not built (reference sources absent)")
    return oracle.Reference()


@pytest.fixture(scope="session")
def gpu_available():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
