"""Writes fq_erf_table.h: for x_i = i/64, i = 0 .. 385 (0 <= x <= 6.016), erf(x_i), erfc(x_i),
G_i = (2/sqrt(pi)) exp(-x_i^2) and the Taylor coefficients q_k = p_k / (k+1), k = 0 .. 15, of
    (erf(x_i + h) - erf(x_i)) / G_i = sum_k q_k h^(k+1),   sum_k p_k h^k = exp(-2 x_i h - h^2),
p_k = (-1)^k H_k(x_i) / k! (Hermite polynomials), from 60-digit mpmath.  Values and q_0 .. q_7 are
double-doubles (hi = the value rounded to double, lo = the rest rounded to double); q_8 .. q_15, whose
terms are below 2^-50 of the sum for |h| <= 1/128, are doubles.  fq_erfinv (fq_math.h) expands erf
around the nearest grid point with them.  Run: python gen_erf_table.py > fq_erf_table.h"""

import sys

import mpmath as mp

mp.mp.dps = 60
N = 386
K = 16
K_DD = 8


def dd(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi.hex(), lo.hex()


def coefficients(x):
    """q_k = (-1)^k H_k(x) / (k! (k+1)), k < K, by the Hermite recurrence in 60 digits."""
    h = [mp.mpf(1), 2 * x]
    for k in range(1, K):
        h.append(2 * x * h[k] - 2 * k * h[k - 1])
    return [(-1) ** k * h[k] / (mp.factorial(k) * (k + 1)) for k in range(K)]


def main(out=sys.stdout):
    two_over_sqrtpi = 2 / mp.sqrt(mp.pi)
    out.write("/* Generated by gen_erf_table.py (mpmath, 60 digits); do not edit.\n")
    out.write(" * Row i (x_i = i / 64): erf(x_i), erfc(x_i), (2/sqrt(pi)) exp(-x_i^2) and q_0 .. q_7 as (hi, lo)\n")
    out.write(" * pairs, then q_8 .. q_15 as doubles: FQ_ERF_ROW doubles per row. */\n")
    out.write("#ifndef FQSB_FQ_ERF_TABLE_H\n#define FQSB_FQ_ERF_TABLE_H\n\n")
    out.write(f"#define FQ_ERF_N {N}\n#define FQ_ERF_K {K}\n#define FQ_ERF_K_DD {K_DD}\n")
    out.write(f"#define FQ_ERF_ROW {6 + 2 * K_DD + (K - K_DD)}\n\n")
    out.write("#define FQ_ERF_TABLE_INIT \\\n    { \\\n")
    for i in range(N):
        x = mp.mpf(i) / 64
        e, c, g = mp.erf(x), mp.erfc(x), two_over_sqrtpi * mp.exp(-x * x)
        q = coefficients(x)
        vals = [*dd(e), *dd(c), *dd(g)]
        for k in range(K_DD):
            vals += dd(q[k])
        vals += [float(q[k]).hex() for k in range(K_DD, K)]
        out.write("        {" + ", ".join(vals) + "}" + (", \\\n" if i + 1 < N else " \\\n"))
    out.write("    }\n\n#endif\n")


if __name__ == "__main__":
    main()
