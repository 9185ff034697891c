import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA kernels)")


@pytest.fixture(scope="session")
def fse():
    """The product package with its CUDA library built in-tree."""
    from falling_sand_engine_gb300 import build

    build.build()
    import falling_sand_engine_gb300 as m

    m.lib()
    m.InitMaterials()
    m.PushMaterials()
    return m


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build_oracle()
    o = oracle.Oracle()
    o.reset_materials()
    return oracle
