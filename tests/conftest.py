import os
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: a CPU test that takes more than a few seconds")


def pytest_sessionstart(session):
    # the product library is built before collection so that tests import a
    # complete extension (a missing build is an error, not a skip)
    import hmpc_gb300

    hmpc_gb300.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def kats():
    import json

    return json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="session")
def cpu_threads():
    return max(1, min(8, os.cpu_count() or 1))
