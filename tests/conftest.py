import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "agilex-7-radar-detect_gb300", ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the CUDA library")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def port():
    import os

    import orc

    # RD_ORACLE_LIB=san: the port built with ASan + UBSan (tests/test_sanitizers.py
    # runs the oracle tests that way in a child process that preloads libasan)
    which = os.environ.get("RD_ORACLE_LIB", "port")
    if not orc.available(which):
        orc.build(which)
    return orc.Oracle(which)


@pytest.fixture(scope="session")
def refo():
    import orc

    if not orc.available("ref"):
        if orc.REF_SOURCES.exists():
            orc.build("ref")
        else:
            pytest.skip("reference sources absent: oracle/_ref not buildable here")
    return orc.Oracle("ref")


@pytest.fixture(scope="session")
def gpulib():
    from rdgb import abi

    lib = abi.load()
    if not lib.rd_device_ok():
        pytest.fail("GPU test without a usable CUDA device")
    return lib


@pytest.fixture(scope="session")
def blockvec():
    import numpy as np

    return np.load(GOLDEN / "block_vectors.npz")


def load_chain_fixture(name):
    import numpy as np

    return np.load(GOLDEN / f"chain_{name}.npz")
