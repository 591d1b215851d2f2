import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The split-precision kernels run every eligible contraction in the tests, the
# small fixtures' too (the library's default sends contractions below 1e7
# flops to the FP64 kernel, where slicing would not pay).
os.environ.setdefault("ITG_SPLIT_MIN_FLOPS", "0")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


def load_golden(name):
    import json
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden():
    return load_golden
