"""In-tree build of the CUDA library (libfqsb.so) for sm_103a.

The translation units compile in parallel with nvcc and are linked into one
shared library under frictionqpotspringblock_gb300/_build/.  Device code is
compiled with -fmad=false and host code with -ffp-contract=off so that no
floating-point expression is contracted into an fma (the kernels also use
explicit rounding intrinsics).
"""

from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = BUILD / "libfqsb.so"
INCLUDE = HERE.parent / "include"
UNITS = ["fqsb_capi.cu", "fqsb_step.cu", "fqsb_noalloc.cu", "fqsb_batch.cu", "fqsb_adjoint.cu", "fqsb_measure.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfqsb.so")


def flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-diag-suppress", "1444",
        "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(INCLUDE),
    ]


def sources() -> list[pathlib.Path]:
    return [CSRC / u for u in UNITS if (CSRC / u).exists()]


def _stale() -> bool:
    if not LIB.exists():
        return True
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    exe = nvcc()
    objs = []

    def compile_one(src: pathlib.Path) -> pathlib.Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [exe] + flags() + ["-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(sources())) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = BUILD / f"libfqsb.{os.getpid()}.so"
    cmd = [exe] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
