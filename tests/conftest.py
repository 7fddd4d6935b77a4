"""Test configuration: paths, the `gpu` marker and shared fixtures.

`-m "not gpu"` runs the oracle known-answer tests, the host-side logic and the
ABI export checks (no GPU needed).  `-m gpu` runs the parity tests of the CUDA
library against the oracle on a GB300.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "tissue-ablation-mc_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def orc():
    import build_oracle

    build_oracle.build()
    import oracle

    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def tam():
    from tam_gb300 import build as b

    if not os.path.exists(b.LIB):
        b.build()
    import tam_gb300

    tam_gb300._abi.load()
    return tam_gb300
