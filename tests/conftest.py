"""Test configuration: the ``gpu`` marker and the build fixtures.

``-m "not gpu"`` runs the oracle, host-logic and library-loading tests on CPU;
``-m gpu`` runs the parity tests, which call the CUDA library through its C ABI
and compare against the CPU oracle on the same inputs.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build_oracle

    build_oracle.build()
    from oracle import oracle

    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    from openmps_gb300 import build

    build.build()
    from openmps_gb300 import computer

    return computer.load_library()
