"""Test configuration: the `gpu` marker and shared builds.

Tests marked `gpu` run the CUDA library on a GPU; the rest run on any CPU
(oracle known answers, NetCDF reader, host logic, C-ABI exports).
"""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle

    pyoracle.build()
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def native():
    from mantaray_gb300 import _native

    return _native.load()
