"""pytest configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs the oracle pins, host logic and ABI checks on any machine; `-m gpu`
runs the CUDA parity tests through the C ABI on a GB300.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def vvlic_lib():
    from vectorvisualization_gb300 import build, capi

    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture()
def ctx(vvlic_lib):
    from vectorvisualization_gb300 import capi

    c = capi.Context(0)
    yield c
    c.close()
