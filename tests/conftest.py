"""Shared fixtures: the CPU restatement (the checker) and, where a GPU is
present, one library context per session."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and the built CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import loader

    loader.build()
    return loader


@pytest.fixture(scope="session")
def ctx():
    import jpxl_gb300 as jg
    from jpxl_gb300 import build

    build.build()
    c = jg.Context(0)
    yield c
    c.close()
