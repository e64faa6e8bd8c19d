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


def test_cpp_header_compiles(tmp_path):
    """include/fqsb.hpp (header-only C++ classes over the C ABI) compiles with every class used."""
    import shutil
    import subprocess

    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = tmp_path / "use_hpp.cpp"
    src.write_text("""
#include "fqsb.hpp"
using namespace FrictionQPotSpringBlock_gb300;
template <class T> void touch(T* s) { if (s) { s->minimise(); s->u(); } }
template <class T> void touch_th(T* s)
{
    if (s) {
        s->flowSteps(10, 0.1);
        auto* e = s->external();
        e->set_state(e->state());
        e->set_next(e->next());
        e->set_f_thermal(e->f_thermal());
    }
}
int main()
{
    touch<Line1d::System_Cuspy_Laplace>(nullptr);
    touch<Line1d::System_SemiSmooth_Laplace>(nullptr);
    touch<Line1d::System_Smooth_Laplace>(nullptr);
    touch<Line1d::System_Cuspy_Laplace_Nopassing>(nullptr);
    touch<Line1d::System_Cuspy_Quartic>(nullptr);
    touch<Line1d::System_Cuspy_QuarticGradient>(nullptr);
    touch<Line1d::System_Cuspy_LongRange>(nullptr);
    touch<Line2d::System_Cuspy_Laplace>(nullptr);
    touch<Line2d::System_Cuspy_QuarticGradient>(nullptr);
    touch<Particles::System_Cuspy>(nullptr);
    touch_th<Line1d::System_Cuspy_Laplace_RandomForcing>(nullptr);
    touch_th<Line1d::System_Cuspy_Quartic_RandomForcing>(nullptr);
    touch_th<Particles::System_Cuspy_RandomForcing>(nullptr);
    return 0;
}
""")
    inc = pathlib.Path(__file__).resolve().parent.parent / "include"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{inc}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
