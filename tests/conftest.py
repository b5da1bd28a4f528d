import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size cases (seconds of oracle time)")


def pytest_collection_modifyitems(config, items):
    # keep the declared file order but make sure test_zz_* files run last
    items.sort(key=lambda it: 1 if Path(str(it.fspath)).name.startswith("test_zz") else 0)
