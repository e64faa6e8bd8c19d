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


def test_c_program_links_and_calls(tmp_path):
    """A plain C caller (the binding a non-Python code base would add) links libfqsb.so, reads the
    version and gets the documented status and message from fqsb_create without a GPU."""
    import shutil
    import subprocess

    import torch

    if shutil.which("gcc") is None:
        pytest.skip("needs gcc")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the program expects FQSB_ERR_NO_DEVICE)")
    from frictionqpotspringblock_gb300 import _build_lib

    lib = _build_lib.build()
    src = tmp_path / "caller.c"
    src.write_text(r"""
#include <stdio.h>
#include <string.h>
#include "fqsb.h"
int main(void)
{
    fqsb_config cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.potential = FQSB_CUSPY; cfg.interactions = FQSB_LAPLACE1D; cfg.rows = 1; cfg.cols = 1024;
    cfg.m = 1; cfg.eta = 0.1; cfg.mu = 1; cfg.k_interactions = 1; cfg.k_frame = 1.0 / 1024; cfg.dt = 0.1;
    cfg.distribution = FQSB_DIST_WEIBULL; cfg.n_parameters = 3;
    cfg.parameters[0] = 2; cfg.parameters[1] = 1; cfg.parameters[2] = 1e-5;
    cfg.offset = -100; cfg.nchunk = 100;
    fqsb_system* h = NULL;
    int rc = fqsb_create(&cfg, &h);
    printf("%s|%d|%s|%d\n", fqsb_version(), rc, fqsb_last_error(NULL), h == NULL);
    return 0;
}
""")
    exe = tmp_path / "caller"
    inc = ROOT / "include"
    r = subprocess.run(["gcc", "-std=c11", f"-I{inc}", str(src), "-o", str(exe), f"-L{lib.parent}", "-lfqsb",
                        f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    version, rc, msg, null = r.stdout.strip().split("|")
    assert version.endswith("sm_103a")
    assert int(rc) == 9 and "no CUDA device" in msg and null == "1"
