"""pytest configuration: the ``gpu`` marker and shared fixtures.

Tests marked ``gpu`` need a CUDA device and the built CUDA library; the CPU
suite (``-m "not gpu"``) covers the oracle against the reference and golden
vectors, host logic, and the C-ABI library's exported symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SCENE_DIR = os.path.join(ROOT, "_scenes")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liblantern_gpu.so")


@pytest.fixture(scope="session")
def scene_dir():
    os.makedirs(SCENE_DIR, exist_ok=True)
    return SCENE_DIR


@pytest.fixture(scope="session")
def reference_available():
    from oracle import oracle as O
    if not os.path.exists(O.REF_SO):
        try:
            O.build_reference()
        except RuntimeError:
            return False
    return os.path.exists(O.REF_SO)
