"""The committed fixtures are what their committed scripts make from the reference tree: the golden
trajectories (tests/golden/make_golden.py, from examples/*.h5) and the API names
(tests/golden/make_api_names.py, from python/main.cpp).  Runs when FQSB_REFERENCE_ROOT names the root of the
reference project (e.g. FQSB_REFERENCE_ROOT=<path> python -m pytest tests/test_fixtures_regenerate.py), else
skipped."""

import importlib.util
import json
import os
import pathlib
import shutil

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).parent / "golden"
REF = pathlib.Path(os.environ.get("FQSB_REFERENCE_ROOT", "")) if os.environ.get("FQSB_REFERENCE_ROOT") else None

pytestmark = pytest.mark.skipif(REF is None or not (REF / "python" / "main.cpp").exists(),
                                reason="FQSB_REFERENCE_ROOT does not name the reference tree")


def _load(name):
    spec = importlib.util.spec_from_file_location(name, GOLDEN / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_golden_trajectories():
    gen = _load("make_golden")
    for stem, (n, first) in gen.FILES.items():
        frame, f_frame, S = gen.read(REF / "examples" / (stem + ".h5"), n, first)
        stored = np.load(GOLDEN / (stem + ".npz"))
        assert np.array_equal(stored["frame"], frame), stem
        assert np.array_equal(stored["f_frame"], f_frame), stem
        assert np.array_equal(stored["S"], S), stem


def test_api_names(tmp_path):
    """make_api_names.py writes next to itself: run a copy in a scratch folder and compare."""
    import sys

    work = tmp_path / "golden"
    work.mkdir()
    shutil.copy(GOLDEN / "make_api_names.py", work / "make_api_names.py")
    spec = importlib.util.spec_from_file_location("make_api_names_copy", work / "make_api_names.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    argv = sys.argv
    try:
        sys.argv = ["make_api_names.py", str(REF)]
        gen.main()
    finally:
        sys.argv = argv
    assert json.loads((work / "api_names.json").read_text()) == json.loads((GOLDEN / "api_names.json").read_text())
