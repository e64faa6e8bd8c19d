"""Integer-pipe binary64 add / sub / mul (frictionqpotspringblock_gb300/csrc/fq_soft64.h).

The step kernels issue part of their fp64 operations through these functions; the parity of the
whole step with the reference rests on each one being bit-identical to the IEEE operation.  The host
check runs the same source against the host's IEEE arithmetic on structured random operands; the
device check compares with the GPU's own fp64 instructions."""

import pathlib
import shutil
import subprocess

import pytest

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE.parent / "frictionqpotspringblock_gb300" / "csrc"


def _build(tmp_path, compiler, src, out, extra):
    exe = tmp_path / out
    subprocess.run([compiler, *extra, f"-I{CSRC}", str(HERE / "soft64" / src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_soft64_host_bit_exact(tmp_path):
    exe = _build(tmp_path, "g++", "soft64_check.cpp", "soft64_check", ["-O2", "-std=c++17", "-ffp-contract=off"])
    r = subprocess.run([str(exe), "2000000", "17"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    fams = {}
    for line in r.stdout.splitlines():
        name, ops, bad, slow = line.split()
        fams[name] = (int(ops), int(bad), int(slow))
    assert all(bad == 0 for _, bad, _ in fams.values())
    # the fast path (not the hardware fallback) carries the bulk of every family but the extremes
    for name in ("raw", "close_exp", "cancel", "ties", "products", "step_regime"):
        ops, _, slow = fams[name]
        assert slow < 0.2 * ops, (name, slow, ops)


@pytest.mark.gpu
def test_soft64_device_bit_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = _build(tmp_path, nvcc, "soft64_device_check.cu", "soft64_device_check",
                 ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-fmad=false"])
    r = subprocess.run([str(exe), "608", "1024"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " mismatches 0 " in r.stdout
