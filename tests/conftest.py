"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built library; the rest run on
CPU only (oracle, host tables, ABI exports, argument validation)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "pr-calc_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libprc_d2z.so")


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(autouse=True)
def _release_device_memory(request):
    """After each GPU test, hand torch's cached device blocks back to the
    driver, so that the next test's free-memory check (the full-size tests
    need 24-110 GB) sees what is really free."""
    yield
    if "gpu" in request.keywords and _have_gpu():
        import gc

        import torch
        gc.collect()
        torch.cuda.empty_cache()
