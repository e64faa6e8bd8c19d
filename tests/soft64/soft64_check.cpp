// Host check of the integer-pipe binary64 add / sub / mul (fq_soft64.h) against the host's IEEE
// arithmetic (compile with -ffp-contract=off).  Usage: soft64_check <cases per family> <seed>.
// Prints one line per input family: name, operations, mismatches, operations that took the hardware
// path; exits 1 on any mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#define FQ_S_COUNT_SLOW 1
#include "fq_soft64.h"

long long fq_s_slow_count = 0;

static const uint64_t MANT52 = 0x000fffffffffffffULL;
static uint64_t g_s;
static uint64_t rnd()
{
    // splitmix64
    uint64_t z = (g_s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static double mk(uint64_t sign, uint64_t e, uint64_t mant)
{
    return fq_from_bits((sign << 63) | ((e & 0x7ff) << 52) | (mant & MANT52));
}
static uint64_t few_bits_mant(int nbits)
{
    // significand with only the top nbits possibly set (exact products / ties)
    uint64_t m = rnd() & MANT52;
    return nbits >= 52 ? m : (m >> (52 - nbits)) << (52 - nbits);
}
static long long g_bad = 0;
static void report(const char* op, double a, double b, double got, double want)
{
    if (g_bad < 10) {
        printf("MISMATCH %s a=%016llx b=%016llx got=%016llx want=%016llx\n", op, (unsigned long long)fq_bits(a),
               (unsigned long long)fq_bits(b), (unsigned long long)fq_bits(got), (unsigned long long)fq_bits(want));
    }
    g_bad++;
}
static bool same(double x, double y)
{
    if (x != x && y != y) {
        return true;
    }
    return fq_bits(x) == fq_bits(y);
}
static void pair(int fam, double& a, double& b)
{
    uint64_t s1 = rnd() & 1, s2 = rnd() & 1;
    switch (fam) {
        case 0: // raw bit patterns
            a = fq_from_bits(rnd());
            b = fq_from_bits(rnd());
            break;
        case 1: { // exponents within 64 of each other, full significands
            uint64_t e1 = 1 + rnd() % 2046;
            int64_t de = (int64_t)(rnd() % 129) - 64;
            int64_t e2 = (int64_t)e1 + de;
            if (e2 < 1) e2 = 1;
            if (e2 > 2046) e2 = 2046;
            a = mk(s1, e1, rnd());
            b = mk(s2, (uint64_t)e2, rnd());
            break;
        }
        case 2: { // near cancellation: b = -a with perturbed low bits / neighbouring exponent
            uint64_t e1 = 1 + rnd() % 2046;
            uint64_t m = rnd();
            a = mk(s1, e1, m);
            uint64_t e2 = e1 + (rnd() % 3) - 1;
            if (e2 < 1 || e2 > 2046) e2 = e1;
            uint64_t m2 = (rnd() & 1) ? (m ^ (rnd() & ((1ULL << (rnd() % 53)) - 1))) : rnd();
            b = mk(s1 ^ 1, e2, m2);
            break;
        }
        case 3: { // few-bit significands: exact halves (ties) and exact results
            uint64_t e1 = 1 + rnd() % 2046;
            int64_t e2 = (int64_t)e1 - (int64_t)(rnd() % 60);
            if (e2 < 1) e2 = 1;
            a = mk(s1, e1, rnd());
            b = mk(s2, (uint64_t)e2, few_bits_mant((int)(rnd() % 8)));
            break;
        }
        case 4: { // extremes: near overflow and near the subnormal boundary, zeros, subnormals, inf, nan
            uint64_t pick[8] = {1, 2, 3, 2045, 2046, 0, 2047, 1 + rnd() % 2046};
            a = mk(s1, pick[rnd() % 8], rnd() & 1 ? rnd() : 0);
            b = mk(s2, pick[rnd() % 8], rnd() & 1 ? rnd() : 0);
            break;
        }
        case 5: { // products: few-bit significands (exact and tie products), exponents near the edges
            int n1 = (int)(rnd() % 53), n2 = (int)(rnd() % 53);
            uint64_t e1 = 1 + rnd() % 2046, e2 = 1 + rnd() % 2046;
            if (rnd() & 1) { // keep the product exponent near the normal range's edges
                int64_t t = (rnd() & 1) ? 1023 + 1023 : 1023 - 1021;
                int64_t x = t - (int64_t)e1 + 1023 + (int64_t)(rnd() % 5) - 2;
                e2 = (uint64_t)(x < 1 ? 1 : (x > 2046 ? 2046 : x));
            }
            a = mk(s1, e1, few_bits_mant(n1));
            b = mk(s2, e2, few_bits_mant(n2));
            break;
        }
        default: { // the step's own regime: positions O(1e3), increments O(1e-5), velocities O(1e-3)
            double u = (double)(int64_t)(rnd() % 20000) - 10000.0 + (double)(rnd() % 1000000) * 1e-6;
            double v = ((double)(rnd() % 2000001) - 1000000.0) * 1e-9;
            a = (rnd() & 1) ? u : v;
            b = (rnd() & 1) ? -u * 0.999999 : v * 0.1;
            break;
        }
    }
}
int main(int argc, char** argv)
{
    long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    g_s = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
    const char* names[7] = {"raw", "close_exp", "cancel", "ties", "extremes", "products", "step_regime"};
    for (int fam = 0; fam < 7; ++fam) {
        long long bad0 = g_bad, slow0 = fq_s_slow_count;
        for (long long i = 0; i < n; ++i) {
            double a, b;
            pair(fam, a, b);
            double r;
            r = fq_sadd(a, b);
            if (!same(r, a + b)) report("add", a, b, r, a + b);
            r = fq_ssub(a, b);
            if (!same(r, a - b)) report("sub", a, b, r, a - b);
            r = fq_smul(a, b);
            if (!same(r, a * b)) report("mul", a, b, r, a * b);
        }
        printf("%s %lld %lld %lld\n", names[fam], 3 * n, g_bad - bad0, fq_s_slow_count - slow0);
    }
    return g_bad ? 1 : 0;
}
