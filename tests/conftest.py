"""Test configuration: the `gpu` marker and shared fixtures.

`-m "not gpu"` runs on any machine (oracle, host logic, library loading);
`-m gpu` needs a GB300 and the library built by __graft_entry__.build().
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def capi():
    from turbulent_lbm_multigpu_gb300 import build, capi as api

    build.build()
    api.lib()
    return api
