"""Shared test set-up: import paths, the `gpu` marker, and session fixtures
that build the GPU library and the oracle once."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("ses3d-nt_gb300", "oracle"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)
if ROOT not in sys.path:
    sys.path.append(ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not _gpu_available():
        pytest.skip("no CUDA GPU")
    return True


@pytest.fixture(scope="session")
def sesnt_lib():
    import sesnt
    lib_path = sesnt.LIB_PATH
    if not os.path.exists(lib_path):
        import build as _b
        _b.build()
    return sesnt.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    import sesnt_oracle
    sesnt_oracle.build()
    return sesnt_oracle
