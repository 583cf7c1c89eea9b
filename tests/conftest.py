import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


# the tile autotuner writes its cache here during the tests (not into $HOME)
os.environ.setdefault("EINSUMS_GB300_AUTOTUNE_CACHE",
                      os.path.join(ROOT, "einsums_gb300", "_build", "autotune_test_cache.txt"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")
