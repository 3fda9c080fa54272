import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "lattice-qcd-rs_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI of liblqgpu.so")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build_oracle, oracle

    build_oracle.build()
    return oracle


@pytest.fixture(scope="session")
def lqgpu_mod():
    import lqgpu_build as lq_build

    lq_build.build()
    import lqgpu

    lqgpu.load()
    return lqgpu
