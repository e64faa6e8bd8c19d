"""The Python API surface against the names the reference binds (python/main.cpp, listed in
tests/golden/api_names.json by tests/golden/make_api_names.py): every submodule and class exists, each
class has exactly the members of the binders the reference applies to it (mySystemNd,
mySystemNdAthermal, mySystemNdDynamics, mySystemNdExternal, main.cpp:46-226) and not those of the
binders it leaves out.  Class attributes only (no instance is created), so this runs without a GPU."""

import json
import pathlib

import pytest

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

NAMES = json.loads((pathlib.Path(__file__).parent / "golden" / "api_names.json").read_text())
SYSTEMS = sorted(k for k, v in NAMES["binders"].items() if v)


def _cls(qualified):
    sub, name = qualified.split(".")
    return getattr(getattr(fqsb, sub), name)


def test_classes():
    for sub, classes in NAMES["classes"].items():
        mod = getattr(fqsb, sub)
        for name in classes:
            assert hasattr(mod, name), f"{sub}.{name}"


@pytest.mark.parametrize("qualified", SYSTEMS)
def test_binders(qualified):
    c = _cls(qualified)
    applied = set(NAMES["binders"][qualified])
    present = {m for b in applied for m in NAMES["binder_members"][b]}
    for m in sorted(present):
        assert hasattr(c, m), m
    for b, members in NAMES["binder_members"].items():
        if b in applied:
            continue
        for m in members:
            if m not in present:
                assert not hasattr(c, m), (b, m)


def test_external_members():
    """detail.RandomNormalForcing_1 (main.cpp:251-275): state, f_thermal, next."""
    c = fqsb.detail.RandomNormalForcing_1
    for m in ("state", "f_thermal", "next"):
        assert hasattr(c, m), m
