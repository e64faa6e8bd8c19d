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


def _check_signature(fn, expected, what):
    import inspect

    params = [p for p in inspect.signature(fn).parameters.values() if p.name != "self"]
    named = [p for p in params if p.kind in (p.POSITIONAL_OR_KEYWORD, p.KEYWORD_ONLY)]
    assert [p.name for p in named[:len(expected)]] == [a for a, _ in expected], what
    for p, (name, default) in zip(named, expected):
        if default is None:
            assert p.default is inspect.Parameter.empty, (what, name)
        else:
            assert p.default == default, (what, name, p.default, default)
    for p in named[len(expected):]:
        assert p.default is not inspect.Parameter.empty, (what, "extra parameter without default", p.name)


@pytest.mark.parametrize("qualified", SYSTEMS)
def test_constructor_arguments(qualified):
    """Argument names, order and defaults of the constructors (py::init bindings of main.cpp)."""
    _check_signature(_cls(qualified).__init__, NAMES["constructors"][qualified], qualified)


@pytest.mark.parametrize("qualified", SYSTEMS)
def test_method_arguments(qualified):
    """Argument names, order and defaults of the bound methods (the binders' py::arg lists)."""
    c = _cls(qualified)
    for b in NAMES["binders"][qualified]:
        for m in NAMES["binder_members"][b]:
            if m in NAMES["methods"] and callable(getattr(c, m, None)) and not isinstance(getattr(c, m), property):
                _check_signature(getattr(c, m), NAMES["methods"][m], f"{qualified}.{m}")
