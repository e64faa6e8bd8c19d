"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports every symbol
declared in include/fqsb.h (no compute call is made without a GPU)."""

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "fqsb.h").read_text()
    return sorted(set(re.findall(r"\b(fqsb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from frictionqpotspringblock_gb300 import _build_lib

    path = _build_lib.build()
    return ctypes.CDLL(str(path))


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from frictionqpotspringblock_gb300 import _capi

    assert sorted(_capi.exported_symbols()) == declared_symbols()


def test_version_string(lib):
    lib.fqsb_version.restype = ctypes.c_char_p
    assert lib.fqsb_version().decode().endswith("sm_103a")


def test_create_without_gpu_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from frictionqpotspringblock_gb300 import Line1d, FrictionError

    with pytest.raises(FrictionError, match="no CUDA device"):
        Line1d.System_Cuspy_Laplace(m=1, eta=1, mu=1, k_interactions=1, k_frame=0.1, dt=1, shape=[5], seed=0,
                                    distribution="delta", parameters=[1.0], offset=-49.5, nchunk=100)
