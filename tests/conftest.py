import os
import sys

import pytest

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)
for _p in (ROOT, TESTS):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAVE_GPU = _cuda_ok()


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle, ozoracle
    build_oracle.build_oracle()
    return ozoracle


@pytest.fixture(scope="session")
def ozlib():
    import ozaie_gb300
    ozaie_gb300.load()
    return ozaie_gb300


@pytest.fixture()
def gpu_handle(ozlib):
    if not HAVE_GPU:
        pytest.skip("no GPU")
    h = ozlib.Handle()
    yield h
    h.close()
