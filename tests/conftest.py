import os
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU run, enabled with FQSB_SLOW=1")


def pytest_collection_modifyitems(config, items):
    # a GPU test that runs away (e.g. a minimise that cannot converge) ends after 5 minutes instead of
    # holding the GPU; needs pytest-timeout (present here and on the GPU hosts), skipped if absent
    if config.pluginmanager.hasplugin("timeout"):
        for item in items:
            if "gpu" in item.keywords and item.get_closest_marker("timeout") is None:
                item.add_marker(pytest.mark.timeout(300))
    if os.environ.get("FQSB_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow; set FQSB_SLOW=1")
    for item in items:
        if "slow" in item.keywords:
            item.add_marker(skip)
