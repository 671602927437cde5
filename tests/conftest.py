import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "spock.cu_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["reftest", "cfg1", "qpl", "affpoly"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def read_bt(path):
    with open(path, "rb") as fh:
        dims = np.frombuffer(fh.read(24), dtype="<u8").astype(np.int64)
        dt = {"d": "<f8", "f": "<f4", "u": "<u8"}[path[-4]]
        a = np.frombuffer(fh.read(), dtype=dt)
    return a, tuple(dims)


def golden(case, name):
    return read_bt(os.path.join(GOLDEN, case, name))[0]


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def tmp_problems(tmp_path_factory):
    return str(tmp_path_factory.mktemp("problems"))
