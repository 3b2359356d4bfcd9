import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels")


def pytest_runtest_setup(item):
    if item.get_closest_marker("gpu") is not None:
        import torch
        if not torch.cuda.is_available():
            pytest.fail("GPU test selected but no CUDA device is visible")


class Golden:
    """Reference outputs recorded by tests/golden/make_golden.py."""

    def __init__(self):
        self.arrays = np.load(GOLDEN / "golden.npz")
        meta = json.loads((GOLDEN / "cases.json").read_text())
        self.cases = meta["cases"]
        self.errors = meta["errors"]

    def __getitem__(self, key):
        return self.arrays[key]

    def of_kind(self, kind):
        return [c for c in self.cases if c["kind"] == kind]

    def state_of(self, case):
        return self.arrays[case.get("state_key", case["name"] + "/state")]


_GOLDEN = None


def golden_data() -> Golden:
    global _GOLDEN
    if _GOLDEN is None:
        _GOLDEN = Golden()
    return _GOLDEN


@pytest.fixture(scope="session")
def golden():
    return golden_data()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib_built():
    from qcware_unitair_gb300 import build_lib
    return build_lib.build()
