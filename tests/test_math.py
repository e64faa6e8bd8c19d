"""The deterministic elementary functions (csrc/fq_math.h) against glibc and high precision.

The device and the oracle's "portable" mode use fq_math.h so that they agree bit for bit; the
reference (prrng, detail.h:406) calls the host libm.  These tests bound the difference between the
two: fq_log / fq_pow / fq_sin are correctly rounded except in rare near-midpoint cases, so they
agree with glibc in (almost) every case and never differ by more than one ulp.
"""

import math

import numpy as np
import pytest

from oracle import oracle as O

mpmath = pytest.importorskip("mpmath")


def ulp_diff(a, b):
    ia = np.array([a], dtype=np.float64).view(np.int64)[0]
    ib = np.array([b], dtype=np.float64).view(np.int64)[0]
    return abs(int(ia) - int(ib))


def test_log_weibull_inputs_agree_with_glibc():
    """x = 1 - u32 * 2^-32, the arguments the weibull / exponential transforms pass to log.

    fq_log and glibc differ by at most one ulp, in about 0.1% of the inputs; in every such case
    fq_log is the correctly rounded value (glibc's log is accurate to ~0.52 ulp, not correctly
    rounded)."""
    mpmath.mp.prec = 200
    rng = np.random.default_rng(0)
    r32 = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64)
    worst, differ = 0, 0
    for r in r32:
        x = 1.0 - float(r) * 2.0 ** -32
        a = O.math("log", x, math_mode=O.MATH_PORTABLE)
        b = O.math("log", x, math_mode=O.MATH_LIBM)
        d = ulp_diff(a, b)
        worst = max(worst, d)
        if d:
            differ += 1
            assert a == float(mpmath.log(mpmath.mpf(x)))
    assert worst <= 1
    assert differ <= 0.005 * len(r32), differ


def test_log_correctly_rounded_sample():
    mpmath.mp.prec = 200
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(1e-12, 1.0, 500), rng.uniform(1.0, 1e6, 500), [0.5, 2.0, 1 - 2 ** -32, 2 ** -32]])
    bad = 0
    for x in xs:
        exact = float(mpmath.log(mpmath.mpf(float(x))))
        bad += O.math("log", float(x)) != exact
    assert bad <= 1, bad


def test_log_special_values():
    assert O.math("log", 1.0) == 0.0
    assert O.math("log", 0.0) == -math.inf
    assert math.isnan(O.math("log", -1.0))
    assert O.math("log", math.inf) == math.inf
    assert abs(O.math("log", 5e-324) - math.log(5e-324)) <= 1e-12


def test_pow_sqrt_branch_is_exact():
    rng = np.random.default_rng(2)
    for x in rng.uniform(0.0, 30.0, 2000):
        assert O.math("pow", float(x), 0.5) == math.sqrt(float(x))


def test_pow_general_exponent():
    mpmath.mp.prec = 200
    rng = np.random.default_rng(3)
    worst = 0
    for x, y in zip(rng.uniform(1e-6, 40.0, 800), rng.uniform(0.1, 3.0, 800)):
        exact = float(mpmath.power(mpmath.mpf(float(x)), mpmath.mpf(float(y))))
        worst = max(worst, ulp_diff(O.math("pow", float(x), float(y)), exact))
    assert worst <= 1


def test_sin_smooth_potential_range():
    """The Smooth potential evaluates sin(pi * (u - u_min) / dy) with |argument| <= pi."""
    mpmath.mp.prec = 200
    rng = np.random.default_rng(4)
    worst, differ = 0, 0
    for x in rng.uniform(-math.pi, math.pi, 4000):
        exact = float(mpmath.sin(mpmath.mpf(float(x))))
        d = ulp_diff(O.math("sin", float(x)), exact)
        worst = max(worst, d)
        differ += d != 0
    assert worst <= 1
    assert differ <= 4, differ


def test_exp():
    mpmath.mp.prec = 200
    rng = np.random.default_rng(5)
    worst = 0
    for x in rng.uniform(-700.0, 700.0, 1000):
        exact = float(mpmath.exp(mpmath.mpf(float(x))))
        worst = max(worst, ulp_diff(O.math("exp", float(x)), exact))
    assert worst <= 1


def test_cos_range():
    mpmath.mp.prec = 200
    rng = np.random.default_rng(6)
    worst = 0
    for x in np.concatenate([rng.uniform(-math.pi, math.pi, 3000), [0.0, math.pi / 2, -math.pi, math.pi]]):
        exact = float(mpmath.cos(mpmath.mpf(float(x))))
        worst = max(worst, ulp_diff(O.math("cos", float(x)), exact))
    assert worst <= 1


def test_erfinv_correctly_rounded():
    """fq_erfinv (the normal quantile of thermal forcing) against 40-digit erfinv on the inputs the
    forcing produces, 2 r - 1 with r = u32 2^-32, and on edge values."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(7)
    r = rng.integers(0, 2 ** 32, 4000, dtype=np.uint64).astype(np.float64) * 2.0 ** -32
    ys = np.concatenate([2 * r - 1, [1e-300, -1e-20, 2.0 ** -52, 0.5, -0.5, 0.999999, 1 - 2.0 ** -31,
                                     -(1 - 2.0 ** -32), 2.0 ** -31 - 1]])
    for y in ys:
        assert O.math("erfinv", float(y)) == float(mp.erfinv(mp.mpf(float(y)))), y
    assert O.math("erfinv", 0.0) == 0.0
    assert O.math("erfinv", 1.0) == np.inf and O.math("erfinv", -1.0) == -np.inf
    assert np.isnan(O.math("erfinv", 1.5))


def test_erfinv_correctly_rounded_whole_domain():
    """fq_erfinv beyond the forcing grid: uniform inputs, 1 - y down to 2^-53 (x up to 5.86, the end of its
    erf table), magnitudes down to the subnormals (the a sqrt(pi)/2 branch below 2^-500), and the
    table's branch points."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(11)
    ys = np.concatenate([rng.uniform(-1, 1, 500), 1 - 10 ** rng.uniform(-16, -1, 500),
                         -(10 ** rng.uniform(-320, -1, 500)),
                         [2.0 ** -500, 2.0 ** -499, 1e-200, 5e-324, 2.2250738585072014e-308, 1 - 2.0 ** -53,
                          0.5, np.nextafter(0.5, 1.0), np.nextafter(0.5, 0.0), 2.0 ** -26]])
    for y in ys:
        assert O.math("erfinv", float(y)) == float(mp.erfinv(mp.mpf(float(y)))), y


def test_erf_table_matches_its_generator():
    """csrc/fq_erf_table.h is exactly what csrc/gen_erf_table.py writes (60-digit mpmath)."""
    pytest.importorskip("mpmath")
    import importlib.util
    import io
    import pathlib

    csrc = pathlib.Path(__file__).resolve().parent.parent / "frictionqpotspringblock_gb300" / "csrc"
    spec = importlib.util.spec_from_file_location("gen_erf_table", csrc / "gen_erf_table.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    out = io.StringIO()
    gen.main(out)
    assert out.getvalue() == (csrc / "fq_erf_table.h").read_text()
