import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "del-msh_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build as obuild
    from oracle import oracle as O
    obuild.build_oracle()
    return O


@pytest.fixture(scope="session")
def golden_dir():
    return ROOT / "tests" / "golden"


@pytest.fixture(scope="session")
def cuda():
    """The CUDA library (built if needed) and torch on cuda:0."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from del_msh_gb300 import _native
    _native.load(build_if_missing=True)
    return torch
