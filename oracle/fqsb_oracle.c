/*
 * CPU oracle for the FrictionQPotSpringBlock time-integration path.
 *
 * TEST INFRASTRUCTURE ONLY (see fqsb_oracle.h).  Every function cites the
 * reference statement it restates; the operation order and association of
 * every floating-point expression follows the reference so that, compiled
 * with -ffp-contract=off, results match the reference's arithmetic.
 *
 * prrng (third-party, pinned in the reference's environment.yaml:13 as
 * prrng >= 1.11.1, absent from the reference tree) is restated here from its
 * published behaviour and its call sites in the reference:
 *   - one pcg32 (O'Neill, XSH-RR 64/32) per particle, seeded with
 *     initstate = seed + p, initseq = 0 (Line1d.h:150-151, Line2d.h:28-34);
 *   - draws mapped to [0,1) as u32 * 2^-32, then the distribution transform;
 *   - the chunk holds the cumulative sum of nchunk draws, shifted once by the
 *     global offset (Line1d.h:157); when a particle leaves the chunk the chunk
 *     is moved and extended by continuing the running sum;
 *   - align(u) gives, per particle, i with y[i] <= u < y[i+1]
 *     (alignment(buffer 2, margin 30, min_margin 6, strict false),
 *     Line1d.h:154).
 * The canonical yield sequence (one definition, independent of where the
 * chunk window sits) is:
 *     0 <= k < nchunk : c_0 = d_0, c_k = c_{k-1} + d_k, y_k = c_k + offset
 *     k >= nchunk     : y_k = y_{k-1} + d_k
 *     k < 0           : y_k = y_{k+1} - d_{k+1}
 * and, after chunk.restore(state, value, index), relative to that anchor:
 *     y_index = value, y_k = y_{k-1} + d_k (k > index), y_k = y_{k+1} - d_{k+1} (k < index).
 */
#include "fqsb_oracle.h"

#include "../frictionqpotspringblock_gb300/csrc/fq_math.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/*
 * Built with -fopenmp (the threaded variant timed as the CPU reference arm), the per-particle loops of
 * construction and of timeStep run in parallel over particle ranges; every iteration is independent
 * (reductions and the thermal draws, which follow one sequential stream, stay sequential), so the
 * results equal the single-threaded build's bit for bit.
 */
#ifdef _OPENMP
#include <omp.h>
#define OQ_PARALLEL_FOR _Pragma("omp parallel for schedule(static)")
static int oq_thread_id(void)
{
    return omp_get_thread_num();
}
static int oq_max_threads(void)
{
    return omp_get_max_threads();
}
#else
#define OQ_PARALLEL_FOR
static int oq_thread_id(void)
{
    return 0;
}
static int oq_max_threads(void)
{
    return 1;
}
#endif

#define PCG_MULT 0x5851f42d4c957f2dULL

struct oq_system {
    int pot, inter;
    int64_t rows, cols, N, n;
    double m, inv_m, eta, mu, kappa, k, k_frame, dt;
    double ia, ib; /* Quartic1d: a1, a2; QuarticGradient1d / 2d: k2, k4; LongRange1d: alpha */
    double* lr_pref; /* LongRange1d: k / d^(alpha + 1) for ring distance d (0 for d = 0) */
    /* RandomNormalForcing (detail.h:881-1000): one pcg32 stream drawn in particle order */
    int thermal, th_mode;
    double th_mean, th_std;
    uint64_t th_state, th_inc;
    int64_t *th_next, *th_dinc;
    double* f_th;
    int64_t lr_m;    /* LongRange1d: the midpoint (N - N % 2) / 2 */
    int dist, npar;
    double par[4];
    double offset;
    double* offp;
    int sum_mode, math_mode;
    int64_t buffer, margin, min_margin;
    /* chunk */
    uint64_t* g0;  /* pcg32 state before draw 0 */
    uint64_t* inc; /* pcg32 increment */
    int* restored;
    int64_t* kr;
    uint64_t* sr;
    double* yr;
    double* data;
    int64_t* start;
    int64_t* cidx;
    /* state (detail.h:1061-1075) */
    double *u, *v, *a, *v_n, *a_n, *f, *f_pot, *f_int, *f_frame, *f_damp;
    double u_frame;
    int64_t inc_n, qs_first, qs_last;
    double* tmp;
    int64_t tmp_n;
    double* blk;
    char err[512];
};

/* ------------------------------------------------------------------ pcg32 */

static inline uint32_t pcg_output(uint64_t old)
{
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

static inline uint64_t pcg_step(uint64_t s, uint64_t inc)
{
    return s * PCG_MULT + inc;
}

/* pcg32_srandom_r: state = 0, inc = 2*initseq+1, step, state += initstate, step. */
static void pcg_seed(uint64_t initstate, uint64_t initseq, uint64_t* state, uint64_t* inc)
{
    *inc = (initseq << 1u) | 1u;
    uint64_t s = 0;
    s = pcg_step(s, *inc);
    s += initstate;
    s = pcg_step(s, *inc);
    *state = s;
}

/* LCG jump-ahead by delta steps (mod 2^64; a negative delta steps back), Brown (1994). */
static uint64_t pcg_advance(uint64_t state, uint64_t inc, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = inc, acc_mult = 1u, acc_plus = 0u;
    while (delta > 0) {
        if (delta & 1u) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    return acc_mult * state + acc_plus;
}

uint32_t oq_pcg32_stream(uint64_t initstate, uint64_t initseq, int64_t n, uint32_t* out)
{
    uint64_t st, inc;
    pcg_seed(initstate, initseq, &st, &inc);
    for (int64_t i = 0; i < n; ++i) {
        out[i] = pcg_output(st);
        st = pcg_step(st, inc);
    }
    return n > 0 ? out[n - 1] : 0;
}

uint64_t oq_pcg32_advance(uint64_t state, uint64_t inc, int64_t delta)
{
    return pcg_advance(state, inc, (uint64_t)delta);
}

/* --------------------------------------------------------- transforms */

static double m_log(double x, int mode)
{
    return mode == OQ_MATH_PORTABLE ? fq_log(x) : log(x);
}

static double m_pow(double x, double y, int mode)
{
    return mode == OQ_MATH_PORTABLE ? fq_pow(x, y) : pow(x, y);
}

static double m_sin(double x, int mode)
{
    return mode == OQ_MATH_PORTABLE ? fq_sin(x) : sin(x);
}

double oq_math(int which, double x, double y, int math_mode)
{
    switch (which) {
        case 0: return m_log(x, math_mode);
        case 1: return m_pow(x, y, math_mode);
        case 2: return m_sin(x, math_mode);
        case 3: return math_mode == OQ_MATH_PORTABLE ? fq_exp(x) : exp(x);
        case 4: return math_mode == OQ_MATH_PORTABLE ? fq_cos(x) : cos(x);
        case 5: return fq_erfinv(x);
        default: return NAN;
    }
}

static double par_or(const double* par, int npar, int i, double def)
{
    return i < npar ? par[i] : def;
}

/*
 * prrng distribution transform of one uniform draw r = u32 * 2^-32 in [0,1).
 * parameters follow prrng: random [scale, offset]; delta [scale, offset];
 * exponential [scale, offset]; power [k, offset]; pareto [k, scale, offset];
 * weibull [k, scale, offset] (test_Line1d.py:285,299 pins the weibull order).
 */
double oq_transform(int dist, const double* par, int npar, uint32_t r32, int mode)
{
    double r = (double)r32 * 0x1p-32;
    switch (dist) {
        case OQ_DIST_RANDOM:
            return r * par_or(par, npar, 0, 1.0) + par_or(par, npar, 1, 0.0);
        case OQ_DIST_DELTA:
            return par_or(par, npar, 0, 1.0) + par_or(par, npar, 1, 0.0);
        case OQ_DIST_EXPONENTIAL:
            return (-m_log(1.0 - r, mode)) * par_or(par, npar, 0, 1.0) + par_or(par, npar, 1, 0.0);
        case OQ_DIST_POWER:
            return m_pow(r, 1.0 / par_or(par, npar, 0, 1.0), mode) + par_or(par, npar, 1, 0.0);
        case OQ_DIST_PARETO:
            return par_or(par, npar, 1, 1.0) / m_pow(1.0 - r, 1.0 / par_or(par, npar, 0, 1.0), mode) +
                   par_or(par, npar, 2, 0.0);
        case OQ_DIST_WEIBULL:
            return par_or(par, npar, 1, 1.0) * m_pow(-m_log(1.0 - r, mode), 1.0 / par_or(par, npar, 0, 1.0), mode) +
                   par_or(par, npar, 2, 0.0);
        default:
            return NAN;
    }
}

static inline double draw(oq_system* s, uint64_t state)
{
    if (s->dist == OQ_DIST_DELTA) {
        return oq_transform(s->dist, s->par, s->npar, 0u, s->math_mode);
    }
    return oq_transform(s->dist, s->par, s->npar, pcg_output(state), s->math_mode);
}

/* ------------------------------------------------- canonical sequence */

static double off_of(oq_system* s, int64_t p)
{
    return s->offp ? s->offp[p] : s->offset;
}

/* y_k for k in [k0, k0+cnt) of particle p, replayed from the particle's anchor. */
static void seq_fill(oq_system* s, int64_t p, int64_t k0, int64_t cnt, double* out)
{
    uint64_t inc = s->inc[p];
    int64_t k1 = k0 + cnt; /* exclusive */
    if (s->restored[p]) {
        int64_t kr = s->kr[p];
        double yr = s->yr[p];
        uint64_t sr = s->sr[p];
        /* forward from the anchor */
        if (k1 > kr) {
            double y = yr;
            uint64_t st = sr;
            if (kr >= k0) {
                out[kr - k0] = y;
            }
            for (int64_t k = kr + 1; k < k1; ++k) {
                st = pcg_step(st, inc);
                y = y + draw(s, st);
                if (k >= k0) {
                    out[k - k0] = y;
                }
            }
        }
        /* backward from the anchor: y_{k} = y_{k+1} - d_{k+1} */
        if (k0 < kr) {
            double y = yr;
            uint64_t st = sr; /* g(k+1) */
            for (int64_t k = kr - 1; k >= k0; --k) {
                y = y - draw(s, st);
                if (k < k1) {
                    out[k - k0] = y;
                }
                st = pcg_advance(st, inc, (uint64_t)(int64_t)-1);
            }
        }
        return;
    }
    int64_t n0 = s->n;
    double o = off_of(s, p);
    uint64_t g0 = s->g0[p];
    if (k1 > 0) {
        uint64_t st = g0;
        double c = 0.0, y = 0.0;
        for (int64_t k = 0; k < k1; ++k) {
            double d = draw(s, st);
            if (k == 0) {
                c = d;
                y = c + o;
            }
            else if (k < n0) {
                c = c + d;
                y = c + o;
            }
            else {
                y = y + d;
            }
            if (k >= k0) {
                out[k - k0] = y;
            }
            st = pcg_step(st, inc);
        }
    }
    if (k0 < 0) {
        double y = draw(s, g0) + o; /* y_0 */
        uint64_t st = g0;           /* g(k+1) */
        for (int64_t k = -1; k >= k0; --k) {
            y = y - draw(s, st);
            if (k < k1) {
                out[k - k0] = y;
            }
            st = pcg_advance(st, inc, (uint64_t)(int64_t)-1);
        }
    }
}

int oq_yield_sequence(oq_system* s, int64_t p, int64_t k0, int64_t count, double* out)
{
    if (p < 0 || p >= s->N || count < 0) {
        return OQ_ERR_INVALID;
    }
    seq_fill(s, p, k0, count, out);
    return OQ_OK;
}

/* prrng align for one particle: y[i] <= u < y[i+1] with the chunk moved when i leaves
 * [min_margin, n - buffer); the moved chunk puts the target at chunk index `margin`. */
static void align_p(oq_system* s, int64_t p, double u)
{
    int64_t n = s->n;
    double* y = s->data + p * n;
    double* blk = s->blk + (size_t)oq_thread_id() * (size_t)n; /* this thread's search block */
    int64_t li = s->cidx[p];
    int64_t gi;
    if (u != u || u == INFINITY || u == -INFINITY) {
        return; /* a NaN is reported by timeStep's check, the index is kept */
    }
    if (y[0] <= u && u < y[n - 1]) {
        if (y[li] <= u) {
            while (li + 1 < n && y[li + 1] <= u) {
                ++li;
            }
        }
        else {
            while (li > 0 && y[li] > u) {
                --li;
            }
        }
        if (li >= s->min_margin && li < n - s->buffer) {
            s->cidx[p] = li;
            return;
        }
        gi = s->start[p] + li;
    }
    else if (u >= y[n - 1]) {
        int64_t k = s->start[p] + n - 1; /* y_k <= u */
        for (;;) {
            seq_fill(s, p, k + 1, n, blk);
            int64_t j = 0;
            while (j < n && blk[j] <= u) {
                ++j;
            }
            if (j < n) {
                gi = k + j;
                break;
            }
            k += n;
        }
    }
    else {
        int64_t k = s->start[p]; /* y_k > u */
        for (;;) {
            seq_fill(s, p, k - n, n, blk);
            int64_t j = n - 1;
            while (j >= 0 && blk[j] > u) {
                --j;
            }
            if (j >= 0) {
                gi = k - n + j;
                break;
            }
            k -= n;
        }
    }
    int64_t ns = gi - s->margin;
    seq_fill(s, p, ns, n, y);
    s->start[p] = ns;
    s->cidx[p] = s->margin;
}

static void align_all(oq_system* s)
{
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < s->N; ++p) {
        align_p(s, p, s->u[p]);
    }
}

/* ------------------------------------------------------------- sums */

static void ensure_tmp(oq_system* s, int64_t n)
{
    if (s->tmp_n < n) {
        free(s->tmp);
        s->tmp = (double*)malloc(sizeof(double) * (size_t)n);
        s->tmp_n = n;
    }
}

/* sum of x[i]*x[i] (square != 0) or of x[i] (square == 0) in the configured order */
static double reduce(oq_system* s, const double* x, int square)
{
    int64_t N = s->N;
    if (s->sum_mode == OQ_SUM_SEQUENTIAL) {
        double r = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            r += square ? x[i] * x[i] : x[i];
        }
        return r;
    }
    int64_t P = 1;
    while (P < N) {
        P *= 2;
    }
    ensure_tmp(s, P + P / 2 + 1);
    double* t = s->tmp;
    OQ_PARALLEL_FOR
    for (int64_t i = 0; i < P; ++i) {
        t[i] = i < N ? (square ? x[i] * x[i] : x[i]) : 0.0;
    }
    /* level by level into the other half of the scratch: within a level every pair is independent,
     * so the threaded build splits the pairs over the threads and keeps the order of additions */
    double* a = t;
    double* b = t + P;
    for (int64_t len = P; len > 1; len /= 2) {
        const int64_t h = len / 2;
        OQ_PARALLEL_FOR
        for (int64_t i = 0; i < h; ++i) {
            b[i] = a[2 * i] + a[2 * i + 1];
        }
        double* c = a;
        a = b;
        b = c;
    }
    return a[0];
}

/* --------------------------------------------------------- forces */

/* Cuspy::force detail.h:139-170, SemiSmooth::force :236-277, Smooth::force :379-409 */
static void compute_force_potential(oq_system* s)
{
    int64_t N = s->N, n = s->n;
    align_all(s);
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        const double* y = s->data + p * n + s->cidx[p];
        double up = s->u[p];
        if (s->pot == OQ_CUSPY) {
            s->f_pot[p] = 0.5 * (y[0] + y[1]) - up;
        }
        else if (s->pot == OQ_SEMISMOOTH) {
            double xi = 0.5 * (y[0] + y[1]);
            double u_r = (s->mu * xi + s->kappa * y[1]) / (s->mu + s->kappa);
            double u_l = (s->mu * xi + s->kappa * y[0]) / (s->mu + s->kappa);
            if (up < u_l) {
                s->f_pot[p] = s->kappa * (up - y[0]);
            }
            else if (up <= u_r) {
                s->f_pot[p] = s->mu * (0.5 * (y[0] + y[1]) - up);
            }
            else {
                s->f_pot[p] = s->kappa * (up - y[1]);
            }
        }
        else {
            double umin = 0.5 * (y[0] + y[1]);
            double dy = 0.5 * (y[1] - y[0]);
            s->f_pot[p] = -s->mu * dy / M_PI * m_sin(M_PI * (up - umin) / dy, s->math_mode);
        }
    }
    if (s->pot == OQ_CUSPY) {
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            s->f_pot[p] *= s->mu;
        }
    }
}

/* Laplace1d::force detail.h:474-487, Laplace2d::force :545-583 */
static void compute_force_interactions(oq_system* s)
{
    int64_t N = s->N;
    const double* u = s->u;
    double* f = s->f_int;
    if (s->inter == OQ_LAPLACE1D) {
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            int64_t l = p == 0 ? N - 1 : p - 1;
            int64_t r = p == N - 1 ? 0 : p + 1;
            f[p] = u[l] - 2 * u[p] + u[r];
        }
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            f[p] *= s->k;
        }
    }
    else if (s->inter == OQ_LONGRANGE1D) {
        /* LongRange1d::force, detail.h:844-866: sequential sum over i != p in index order (before
         * oq_set_interaction_parameters gives alpha the interaction is off) */
        for (int64_t p = 0; p < N && s->lr_pref; ++p) {
            double fp = 0.0;
            double up = u[p];
            for (int64_t i = 0; i < N; ++i) {
                if (i == p) {
                    continue;
                }
                int64_t d = i > p ? i - p : p - i;
                if (d > s->lr_m) {
                    d = N - d;
                }
                fp += (u[i] - up) * s->lr_pref[d];
            }
            f[p] = fp;
        }
    }
    else if (s->inter == OQ_QUARTIC1D) {
        /* Quartic1d::force, detail.h:781-803 */
        for (int64_t p = 0; p < N; ++p) {
            int64_t l = p == 0 ? N - 1 : p - 1;
            int64_t r = p == N - 1 ? 0 : p + 1;
            double dup = u[r] - u[p];
            double dun = u[l] - u[p];
            f[p] = s->ia * (u[l] - 2 * u[p] + u[r]) + s->ib * (dup * dup * dup + dun * dun * dun);
        }
    }
    else if (s->inter == OQ_QUARTICGRAD1D) {
        /* QuarticGradient1d::force, detail.h:636-650 (m_k4_4 = 0.25 * k4, :633) */
        double k4_4 = 0.25 * s->ib;
        for (int64_t p = 0; p < N; ++p) {
            int64_t l = p == 0 ? N - 1 : p - 1;
            int64_t r = p == N - 1 ? 0 : p + 1;
            double du = u[r] - u[l];
            f[p] = (u[l] - 2 * u[p] + u[r]) * (s->ia + k4_4 * du * du);
        }
    }
    else if (s->inter == OQ_QUARTICGRAD2D) {
        /* QuarticGradient2d::force, detail.h:677-750 (periodic neighbours) */
        int64_t R = s->rows, C = s->cols;
        double mk4_3 = s->ib / 3.0;
        double mk4_23 = 2.0 * mk4_3;
        for (int64_t i = 0; i < R; ++i) {
            int64_t im = (i + R - 1) % R, ip = (i + 1) % R;
            for (int64_t j = 0; j < C; ++j) {
                int64_t jm = (j + C - 1) % C, jp = (j + 1) % C;
                double c = u[i * C + j];
                double l = u[ip * C + j] + u[im * C + j] + u[i * C + jp] + u[i * C + jm] - 4 * c;
                double dudx = 0.5 * (u[ip * C + j] - u[im * C + j]);
                double dudy = 0.5 * (u[i * C + jp] - u[i * C + jm]);
                double d2udxdy = 0.25 * (u[ip * C + jp] - u[ip * C + jm] - u[im * C + jp] + u[im * C + jm]);
                double d2udx2 = u[ip * C + j] - 2 * c + u[im * C + j];
                double d2udy2 = u[i * C + jp] - 2 * c + u[i * C + jm];
                f[i * C + j] = l * (s->ia + mk4_3) +
                               mk4_23 * (dudx * dudx * d2udx2 + dudy * dudy * d2udy2 + 2.0 * dudx * dudy * d2udxdy);
            }
        }
    }
    else if (s->inter == OQ_LAPLACE2D) {
        int64_t R = s->rows, C = s->cols;
        OQ_PARALLEL_FOR
        for (int64_t i = 0; i < R; ++i) {
            int64_t im = (i + R - 1) % R, ip = (i + 1) % R;
            for (int64_t j = 0; j < C; ++j) {
                int64_t jm = (j + C - 1) % C, jp = (j + 1) % C;
                f[i * C + j] = u[im * C + j] + u[ip * C + j] + u[i * C + jm] + u[i * C + jp] - 4 * u[i * C + j];
            }
        }
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            f[p] *= s->k;
        }
    }
}

/* computeForceFrame detail.h:1353-1356 */
static void compute_force_frame(oq_system* s)
{
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < s->N; ++p) {
        s->f_frame[p] = s->k_frame * (s->u_frame - s->u[p]);
    }
}

/* computeForceDamping detail.h:1361-1364 */
static void compute_force_damping(oq_system* s)
{
    double me = -s->eta;
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < s->N; ++p) {
        s->f_damp[p] = me * s->v[p];
    }
}

/* computeForce detail.h:1321-1330 (with External: + f_thermal) */
static void compute_force(oq_system* s)
{
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < s->N; ++p) {
        s->f[p] = s->f_frame[p] + s->f_pot[p] + s->f_int[p] + s->f_damp[p];
    }
    if (s->thermal) {
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < s->N; ++p) {
            s->f[p] = s->f[p] + s->f_th[p];
        }
    }
}

static double thermal_draw(oq_system* s)
{
    uint64_t old = s->th_state;
    s->th_state = old * PCG_MULT + s->th_inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    uint32_t u32 = (xs >> rot) | (xs << ((-rot) & 31));
    double r = (double)u32 * 0x1p-32;
    double z = fq_erfinv(2.0 * r - 1.0);
    if (s->th_mode == 1) {
        return s->th_mean + s->th_std * (M_SQRT2 * z);
    }
    return s->th_mean + (s->th_std * M_SQRT2) * z;
}

/* updated_inc detail.h:1369-1375 with RandomNormalForcing::force detail.h:930-942 */
static void updated_inc(oq_system* s)
{
    if (!s->thermal) {
        return;
    }
    for (int64_t p = 0; p < s->N; ++p) {
        if (s->inc_n >= s->th_next[p]) {
            s->f_th[p] = thermal_draw(s);
            s->th_next[p] += s->th_dinc[p];
        }
    }
    compute_force(s);
}

/* updated_u detail.h:1380-1386 */
static void updated_u(oq_system* s)
{
    compute_force_potential(s);
    compute_force_interactions(s);
    compute_force_frame(s);
    compute_force(s);
}

/* updated_v detail.h:1391-1395 */
static void updated_v(oq_system* s)
{
    compute_force_damping(s);
    compute_force(s);
}

/* parameters of the Quartic interactions (System_Cuspy_Quartic / _QuarticGradient constructors) */
int oq_set_interaction_parameters(oq_system* s, double a, double b)
{
    s->ia = a;
    s->ib = b;
    if (s->inter == OQ_LONGRANGE1D) {
        /* LongRange1d constructor, detail.h:828-841 (alpha = a, k = k_interactions, std::pow) */
        int64_t n = s->N;
        free(s->lr_pref);
        s->lr_pref = (double*)malloc(sizeof(double) * (size_t)n);
        s->lr_m = (n - n % 2) / 2;
        for (int64_t d = 0; d < n; ++d) {
            s->lr_pref[d] = d == 0 ? 0.0 : s->k / pow((double)d, a + 1.0);
        }
    }
    return oq_refresh(s);
}

/* ------------------------------------------------------- lifecycle */

static int dist_supported(int dist)
{
    return dist == OQ_DIST_RANDOM || dist == OQ_DIST_DELTA || dist == OQ_DIST_EXPONENTIAL ||
           dist == OQ_DIST_POWER || dist == OQ_DIST_PARETO || dist == OQ_DIST_WEIBULL;
}

oq_system* oq_create(int potential, int interactions, int64_t rows, int64_t cols, double m, double eta, double mu,
                     double kappa, double k_interactions, double k_frame, double dt, uint64_t seed, int distribution,
                     const double* parameters, int n_parameters, double offset, const double* offset_per_particle,
                     int64_t nchunk, int sum_mode, int math_mode)
{
    if (!dist_supported(distribution) || nchunk < 34 || rows < 1 || cols < 1 || n_parameters > 4) {
        return NULL;
    }
    oq_system* s = (oq_system*)calloc(1, sizeof(oq_system));
    s->pot = potential;
    s->inter = interactions;
    s->rows = rows;
    s->cols = cols;
    s->N = rows * cols;
    s->n = nchunk;
    s->m = m;
    s->inv_m = 1.0 / m;
    s->eta = eta;
    s->mu = mu;
    s->kappa = kappa;
    s->k = k_interactions;
    s->k_frame = k_frame;
    s->dt = dt;
    s->dist = distribution;
    s->npar = n_parameters;
    for (int i = 0; i < n_parameters; ++i) {
        s->par[i] = parameters[i];
    }
    s->offset = offset;
    s->sum_mode = sum_mode;
    s->math_mode = math_mode;
    s->buffer = 2;
    s->margin = 30;
    s->min_margin = 6;
    int64_t N = s->N;
    if (offset_per_particle) {
        s->offp = (double*)malloc(sizeof(double) * (size_t)N);
        memcpy(s->offp, offset_per_particle, sizeof(double) * (size_t)N);
    }
    s->g0 = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)N);
    s->inc = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)N);
    s->restored = (int*)calloc((size_t)N, sizeof(int));
    s->kr = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    s->sr = (uint64_t*)calloc((size_t)N, sizeof(uint64_t));
    s->yr = (double*)calloc((size_t)N, sizeof(double));
    s->data = (double*)malloc(sizeof(double) * (size_t)(N * nchunk));
    s->start = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    s->cidx = (int64_t*)calloc((size_t)N, sizeof(int64_t));
    s->blk = (double*)malloc(sizeof(double) * (size_t)nchunk * (size_t)oq_max_threads());
    double** arrs[] = {&s->u, &s->v, &s->a, &s->v_n, &s->a_n, &s->f, &s->f_pot, &s->f_int, &s->f_frame, &s->f_damp};
    for (size_t i = 0; i < sizeof(arrs) / sizeof(arrs[0]); ++i) {
        *arrs[i] = (double*)calloc((size_t)N, sizeof(double));
    }
    /* Generator(initstate = seed + arange(N), initseq = 0), Line1d.h:148-155; Line2d.h:28-34 */
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        pcg_seed(seed + (uint64_t)p, 0u, &s->g0[p], &s->inc[p]);
        seq_fill(s, p, 0, nchunk, s->data + p * nchunk);
    }
    /* initSystem detail.h:1096-1139 */
    s->u_frame = 0.0;
    oq_refresh(s);
    return s;
}

void oq_destroy(oq_system* s)
{
    if (!s) {
        return;
    }
    free(s->offp);
    free(s->g0);
    free(s->inc);
    free(s->restored);
    free(s->kr);
    free(s->sr);
    free(s->yr);
    free(s->data);
    free(s->start);
    free(s->cidx);
    free(s->blk);
    free(s->u);
    free(s->v);
    free(s->a);
    free(s->v_n);
    free(s->a_n);
    free(s->f);
    free(s->f_pot);
    free(s->f_int);
    free(s->f_frame);
    free(s->f_damp);
    free(s->tmp);
    free(s->lr_pref);
    free(s->th_next);
    free(s->th_dinc);
    free(s->f_th);
    free(s);
}

const char* oq_last_error(oq_system* s)
{
    return s->err;
}

int64_t oq_size(oq_system* s)
{
    return s->N;
}

static int fail(oq_system* s, int code, const char* msg)
{
    snprintf(s->err, sizeof(s->err), "%s", msg);
    return code;
}

/* ------------------------------------------------------ accessors */

static double* field_ptr(oq_system* s, int field)
{
    switch (field) {
        case OQ_F_U: return s->u;
        case OQ_F_V: return s->v;
        case OQ_F_A: return s->a;
        case OQ_F_F: return s->f;
        case OQ_F_F_POTENTIAL: return s->f_pot;
        case OQ_F_F_INTERACTIONS: return s->f_int;
        case OQ_F_F_FRAME: return s->f_frame;
        case OQ_F_F_DAMPING: return s->f_damp;
        default: return NULL;
    }
}

int oq_get(oq_system* s, int field, double* out)
{
    double* p = field_ptr(s, field);
    if (!p) {
        return OQ_ERR_INVALID;
    }
    memcpy(out, p, sizeof(double) * (size_t)s->N);
    return OQ_OK;
}

/* set_u detail.h:1231-1236, set_v :1244-1249, set_a :1255-1259 */
int oq_set(oq_system* s, int field, const double* in)
{
    double* p = field_ptr(s, field);
    if (!p || field > OQ_F_A) {
        return OQ_ERR_INVALID;
    }
    memcpy(p, in, sizeof(double) * (size_t)s->N);
    if (field == OQ_F_U) {
        updated_u(s);
    }
    else if (field == OQ_F_V) {
        updated_v(s);
    }
    return OQ_OK;
}

/* residual detail.h:1512-1520 */
static double residual(oq_system* s)
{
    double r_fres = sqrt(reduce(s, s->f, 1));
    double r_fext = sqrt(reduce(s, s->f_frame, 1));
    if (r_fext != 0.0) {
        return r_fres / r_fext;
    }
    return r_fres;
}

double oq_get_scalar(oq_system* s, int which)
{
    switch (which) {
        case OQ_S_U_FRAME: return s->u_frame;
        case OQ_S_T: return (double)s->inc_n * s->dt; /* t detail.h:1484-1487 */
        case OQ_S_TEMPERATURE: return 0.5 * s->m * reduce(s, s->v, 1) / (double)s->N; /* :1500-1503 */
        case OQ_S_RESIDUAL: return residual(s);
        case OQ_S_MEAN_F_FRAME: return reduce(s, s->f_frame, 0) / (double)s->N;
        default: return NAN;
    }
}

/* set_u_frame detail.h:1253-1258: f_frame and f are updated, a is not */
int oq_set_u_frame(oq_system* s, double v)
{
    s->u_frame = v;
    compute_force_frame(s);
    compute_force(s);
    return OQ_OK;
}

/* set_inc detail.h:1212-1218 */
int oq_set_inc(oq_system* s, int64_t inc)
{
    s->inc_n = inc;
    s->qs_first = inc;
    s->qs_last = inc;
    compute_force(s);
    updated_inc(s);
    return OQ_OK;
}

/*
 * Attach a RandomNormalForcing (Line1d.h:264-330): mean, stddev, the pcg32 (state, inc) after
 * seeding, per-particle first increment `next` and interval `dinc`; then updated_inc as initSystem's
 * refresh does (detail.h:1310-1315).  `mode` selects the normal transform's association (exploratory:
 * prrng's normal transform is not in the reference tree).
 */
int oq_set_thermal(oq_system* s, double mean, double stddev, uint64_t state, uint64_t inc, const int64_t* next,
                   const int64_t* dinc, int mode)
{
    int64_t N = s->N;
    s->thermal = 1;
    s->th_mode = mode;
    s->th_mean = mean;
    s->th_std = stddev;
    s->th_state = state;
    s->th_inc = inc;
    free(s->th_next);
    free(s->th_dinc);
    free(s->f_th);
    s->th_next = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    s->th_dinc = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    s->f_th = (double*)calloc((size_t)N, sizeof(double));
    memcpy(s->th_next, next, sizeof(int64_t) * (size_t)N);
    memcpy(s->th_dinc, dinc, sizeof(int64_t) * (size_t)N);
    updated_inc(s);
    return OQ_OK;
}

int oq_thermal_get(oq_system* s, uint64_t* state, double* f_thermal, int64_t* next)
{
    if (!s->thermal) {
        return fail(s, OQ_ERR_INVALID, "no RandomNormalForcing attached");
    }
    if (state) {
        *state = s->th_state;
    }
    if (f_thermal) {
        memcpy(f_thermal, s->f_th, sizeof(double) * (size_t)s->N);
    }
    if (next) {
        memcpy(next, s->th_next, sizeof(int64_t) * (size_t)s->N);
    }
    return OQ_OK;
}

/* set_state (prrng restore: the state, the stream kept), set_f_thermal, set_next: detail.h:956-995 */
int oq_thermal_set(oq_system* s, const uint64_t* state, const double* f_thermal, const int64_t* next)
{
    if (!s->thermal) {
        return fail(s, OQ_ERR_INVALID, "no RandomNormalForcing attached");
    }
    if (state) {
        s->th_state = *state;
    }
    if (f_thermal) {
        memcpy(s->f_th, f_thermal, sizeof(double) * (size_t)s->N);
    }
    if (next) {
        memcpy(s->th_next, next, sizeof(int64_t) * (size_t)s->N);
    }
    return OQ_OK;
}

int oq_get_thermal(oq_system* s, double* f_thermal)
{
    if (!s->thermal) {
        return fail(s, OQ_ERR_INVALID, "no RandomNormalForcing attached");
    }
    memcpy(f_thermal, s->f_th, sizeof(double) * (size_t)s->N);
    return OQ_OK;
}

int64_t oq_get_inc(oq_system* s)
{
    return s->inc_n;
}

/* set_t detail.h:1200-1204 */
int oq_set_t(oq_system* s, double t)
{
    s->inc_n = (int64_t)round(t / s->dt);
    return OQ_OK;
}

int oq_get_index(oq_system* s, int64_t* gidx, int64_t* cidx, double* left, double* right)
{
    for (int64_t p = 0; p < s->N; ++p) {
        int64_t c = s->cidx[p];
        if (gidx) {
            gidx[p] = s->start[p] + c;
        }
        if (cidx) {
            cidx[p] = c;
        }
        if (left) {
            left[p] = s->data[p * s->n + c];
        }
        if (right) {
            right[p] = s->data[p * s->n + c + 1];
        }
    }
    return OQ_OK;
}

int oq_chunk_data(oq_system* s, double* out, int64_t* start)
{
    if (out) {
        memcpy(out, s->data, sizeof(double) * (size_t)(s->N * s->n));
    }
    if (start) {
        memcpy(start, s->start, sizeof(int64_t) * (size_t)s->N);
    }
    return OQ_OK;
}

/* pcg32 state such that the next draw gives the draw of global index `index` */
int oq_chunk_state_at(oq_system* s, const int64_t* index, uint64_t* state)
{
    for (int64_t p = 0; p < s->N; ++p) {
        if (s->restored[p]) {
            state[p] = pcg_advance(s->sr[p], s->inc[p], (uint64_t)(index[p] - s->kr[p]));
        }
        else {
            state[p] = pcg_advance(s->g0[p], s->inc[p], (uint64_t)index[p]);
        }
    }
    return OQ_OK;
}

/* prrng chunk.restore(state, value, index): the chunk restarts at `index` with data[0] = value */
int oq_chunk_restore(oq_system* s, const uint64_t* state, const double* value, const int64_t* index)
{
    for (int64_t p = 0; p < s->N; ++p) {
        s->restored[p] = 1;
        s->kr[p] = index[p];
        s->sr[p] = state[p];
        s->yr[p] = value[p];
        s->start[p] = index[p];
        s->cidx[p] = 0;
        seq_fill(s, p, index[p], s->n, s->data + p * s->n);
    }
    return OQ_OK;
}

int64_t oq_quasistatic_first(oq_system* s)
{
    return s->qs_first;
}

int64_t oq_quasistatic_last(oq_system* s)
{
    return s->qs_last;
}

/* ------------------------------------------------------- dynamics */

/* refresh detail.h:1310-1315 */
int oq_refresh(oq_system* s)
{
    updated_u(s);
    updated_v(s);
    compute_force(s);
    updated_inc(s);
    return OQ_OK;
}

/* quench detail.h:1527-1532 */
int oq_quench(oq_system* s)
{
    memset(s->v, 0, sizeof(double) * (size_t)s->N);
    memset(s->a, 0, sizeof(double) * (size_t)s->N);
    updated_v(s);
    return OQ_OK;
}

/* timeStep detail.h:1539-1570 */
int oq_time_step(oq_system* s)
{
    int64_t N = s->N;
    double dt = s->dt, hdt = 0.5 * dt, hdt2 = 0.5 * dt * dt;
    s->inc_n++;
    updated_inc(s);
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        s->v_n[p] = s->v[p];
        s->a_n[p] = s->a[p];
    }
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        s->u[p] = s->u[p] + dt * s->v[p] + hdt2 * s->a[p];
    }
    updated_u(s);
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        s->v[p] = s->v_n[p] + dt * s->a_n[p];
    }
    updated_v(s);
    OQ_PARALLEL_FOR
    for (int64_t p = 0; p < N; ++p) {
        s->a[p] = s->f[p] * s->inv_m;
    }
    for (int rep = 0; rep < 2; ++rep) {
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            s->v[p] = s->v_n[p] + hdt * (s->a_n[p] + s->a[p]);
        }
        updated_v(s);
        OQ_PARALLEL_FOR
        for (int64_t p = 0; p < N; ++p) {
            s->a[p] = s->f[p] * s->inv_m;
        }
    }
    int nan = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : nan)
#endif
    for (int64_t p = 0; p < N; ++p) {
        nan |= isnan(s->u[p]) ? 1 : 0;
    }
    if (nan) {
        return fail(s, OQ_ERR_NAN, "NaN entries found");
    }
    return OQ_OK;
}

/* timeSteps detail.h:1577-1583 */
int oq_time_steps(oq_system* s, uint64_t n)
{
    for (uint64_t i = 0; i < n; ++i) {
        int r = oq_time_step(s);
        if (r) {
            return r;
        }
    }
    return OQ_OK;
}

/* flowSteps detail.h:1637-1645 */
int oq_flow_steps(oq_system* s, uint64_t n, double v_frame)
{
    for (uint64_t i = 0; i < n; ++i) {
        s->u_frame += v_frame * s->dt;
        int r = oq_time_step(s);
        if (r) {
            return r;
        }
    }
    return OQ_OK;
}

/* GooseFEM::Iterate::StopList: rolling window of the last n residuals, initialised to +inf */
typedef struct {
    double* r;
    uint64_t n;
} stoplist;

static void sl_init(stoplist* l, uint64_t n)
{
    l->n = n;
    l->r = (double*)malloc(sizeof(double) * (size_t)(n ? n : 1));
    for (uint64_t i = 0; i < n; ++i) {
        l->r[i] = INFINITY;
    }
}

static void sl_insert(stoplist* l, double v)
{
    if (l->n == 0) {
        return;
    }
    memmove(l->r, l->r + 1, sizeof(double) * (size_t)(l->n - 1));
    l->r[l->n - 1] = v;
}

/* std::is_sorted(begin, end, std::greater<double>()) */
static int sl_descending(const stoplist* l)
{
    for (uint64_t i = 1; i < l->n; ++i) {
        if (l->r[i] > l->r[i - 1]) {
            return 0;
        }
    }
    return 1;
}

static int sl_all_less(const stoplist* l, double tol)
{
    for (uint64_t i = 0; i < l->n; ++i) {
        if (l->r[i] >= tol) {
            return 0;
        }
    }
    return 1;
}

static void gidx_all(oq_system* s, int64_t* out)
{
    for (int64_t p = 0; p < s->N; ++p) {
        out[p] = s->start[p] + s->cidx[p];
    }
}

/* timeStepsUntilEvent detail.h:1595-1622 */
int oq_time_steps_until_event(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, uint64_t* ret)
{
    double tol2 = tol * tol;
    stoplist res;
    sl_init(&res, niter_tol);
    int64_t N = s->N;
    int64_t* i_n = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    gidx_all(s, i_n);
    uint64_t step;
    int rc = OQ_OK;
    for (step = 1; step < max_iter + 1; ++step) {
        rc = oq_time_step(s);
        if (rc) {
            break;
        }
        gidx_all(s, cur);
        int changed = 0;
        for (int64_t p = 0; p < N; ++p) {
            if (cur[p] != i_n[p]) {
                changed = 1;
                break;
            }
        }
        if (changed) {
            goto done;
        }
        sl_insert(&res, residual(s));
        if ((sl_descending(&res) && sl_all_less(&res, tol)) || sl_all_less(&res, tol2)) {
            oq_quench(s);
            step = 0;
            goto done;
        }
    }
done:
    *ret = step;
    free(i_n);
    free(cur);
    free(res.r);
    return rc;
}

static int minimise_impl(oq_system* s, const int64_t* i_n_given, uint64_t A_truncate, uint64_t S_truncate, double tol,
                         uint64_t niter_tol, uint64_t max_iter, int time_activity, int max_iter_is_error, int truncate,
                         uint64_t* ret)
{
    double tol2 = tol * tol;
    stoplist res;
    sl_init(&res, niter_tol);
    int64_t N = s->N;
    int64_t* i_n = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    if (i_n_given) {
        memcpy(i_n, i_n_given, sizeof(int64_t) * (size_t)N);
    }
    else {
        gidx_all(s, i_n);
    }
    long sum_s = 0, s_n = 0;
    int init = 1;
    uint64_t step;
    int rc = OQ_OK;
    for (step = 1; step < max_iter + 1; ++step) {
        rc = oq_time_step(s);
        if (rc) {
            goto out;
        }
        sl_insert(&res, residual(s));
        uint64_t a = 0;
        if (time_activity || truncate) {
            gidx_all(s, cur);
            sum_s = 0;
            for (int64_t p = 0; p < N; ++p) {
                int64_t d = cur[p] - i_n[p];
                sum_s += d < 0 ? -d : d;
                a += cur[p] != i_n[p];
            }
            if (sum_s != s_n) {
                if (init) {
                    init = 0;
                    s->qs_first = s->inc_n;
                }
                s->qs_last = s->inc_n;
            }
            s_n = sum_s;
        }
        if ((sl_descending(&res) && sl_all_less(&res, tol)) || sl_all_less(&res, tol2)) {
            oq_quench(s);
            *ret = 0;
            goto out;
        }
        if (truncate) {
            if (A_truncate > 0 && a >= A_truncate) {
                *ret = step;
                goto out;
            }
            if (S_truncate > 0 && sum_s >= (long)S_truncate) {
                *ret = step;
                goto out;
            }
        }
    }
    *ret = step;
    if (max_iter_is_error) {
        rc = fail(s, OQ_ERR_NO_CONVERGENCE, "No convergence found");
    }
out:
    free(i_n);
    free(cur);
    free(res.r);
    return rc;
}

/* minimise detail.h:1676-1792 (generic branch :1754-1785) */
int oq_minimise(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                int max_iter_is_error, uint64_t* ret)
{
    return minimise_impl(s, NULL, 0, 0, tol, niter_tol, max_iter, time_activity, max_iter_is_error, 0, ret);
}

/* minimise_truncate detail.h:1833-1893 */
int oq_minimise_truncate(oq_system* s, const int64_t* i_n, uint64_t A_truncate, uint64_t S_truncate, double tol,
                         uint64_t niter_tol, uint64_t max_iter, int time_activity, int max_iter_is_error, uint64_t* ret)
{
    (void)time_activity;
    return minimise_impl(s, i_n, A_truncate, S_truncate, tol, niter_tol, max_iter, 1, max_iter_is_error, 1, ret);
}

/*
 * minimise of System_Cuspy_Laplace_Nopassing, the Overdamped branch of detail.h:1694-1753 (class
 * Line1d.h:173-238): a Jacobi fixed point over the particles.  From the snapshot v_n = u of the
 * previous sweep, each particle takes the position that balances its neighbours' springs, the frame
 * spring and the parabola of its current well,
 *     u = ((k * (v_n[p-1] + v_n[p+1]) + k_frame * u_frame) + mu * umin) / ((2 * k + k_frame) + mu),
 * with umin the well's centre 0.5 * (y_i + y_{i+1}); the chunk is aligned at u and, while the local
 * chunk index changes, the position is recomputed with the new well.  Then f_frame, f_potential
 * (per particle), f_interactions (after the sweep) and f = (f_potential + f_interactions) + f_frame,
 * and the StopList residual test; quench on convergence.  Time (inc) does not advance.
 */
int oq_minimise_nopassing(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, int max_iter_is_error,
                          uint64_t* ret)
{
    if (s->pot != OQ_CUSPY || s->inter != OQ_LAPLACE1D || s->N < 2) {
        return fail(s, OQ_ERR_INVALID, "the no-passing minimiser needs the Cuspy potential on a Line1d ring, N >= 2");
    }
    double tol2 = tol * tol;
    stoplist res;
    sl_init(&res, niter_tol);
    const int64_t N = s->N, n = s->n;
    const double k = s->k;
    const double den = 2 * k + s->k_frame + s->mu;
    s->qs_first = s->inc_n;
    s->qs_last = s->inc_n;
    uint64_t step;
    int rc = OQ_OK;
    for (step = 1; step < max_iter + 1; ++step) {
        memcpy(s->v_n, s->u, sizeof(double) * (size_t)N);
        for (int64_t p = 0; p < N; ++p) {
            double uneigh;
            if (p == 0) {
                uneigh = s->v_n[N - 1] + s->v_n[1];
            }
            else if (p == N - 1) {
                uneigh = s->v_n[N - 2] + s->v_n[0];
            }
            else {
                uneigh = s->v_n[p - 1] + s->v_n[p + 1];
            }
            int64_t i = s->cidx[p];
            const double* y = s->data + p * n;
            double umin, u;
            for (;;) {
                umin = 0.5 * (y[i] + y[i + 1]);
                u = (k * uneigh + s->k_frame * s->u_frame + s->mu * umin) / den;
                align_p(s, p, u);
                int64_t j = s->cidx[p];
                if (j == i) {
                    break;
                }
                i = j;
            }
            s->u[p] = u;
            s->f_frame[p] = s->k_frame * (s->u_frame - u);
            s->f_pot[p] = s->mu * (umin - u);
        }
        compute_force_interactions(s);
        for (int64_t p = 0; p < N; ++p) {
            s->f[p] = s->f_pot[p] + s->f_int[p] + s->f_frame[p];
        }
        sl_insert(&res, residual(s));
        if ((sl_descending(&res) && sl_all_less(&res, tol)) || sl_all_less(&res, tol2)) {
            oq_quench(s);
            *ret = 0;
            goto out;
        }
    }
    *ret = step;
    if (max_iter_is_error) {
        rc = fail(s, OQ_ERR_NO_CONVERGENCE, "No convergence found");
    }
out:
    free(res.r);
    return rc;
}

/* maxUniformDisplacement detail.h:1901-1905; Cuspy :176-187; SemiSmooth :282-334; Smooth :414-422 */
int oq_max_uniform_displacement(oq_system* s, int direction, double* ret)
{
    int64_t N = s->N, n = s->n;
    if (s->pot == OQ_SMOOTH) {
        return fail(s, OQ_ERR_NOT_POSSIBLE, "Operation not possible.");
    }
    align_all(s);
    double best = INFINITY;
    for (int64_t p = 0; p < N; ++p) {
        const double* y = s->data + p * n + s->cidx[p];
        double up = s->u[p];
        double du;
        if (s->pot == OQ_CUSPY) {
            du = direction > 0 ? y[1] - up : up - y[0];
        }
        else {
            double xi = 0.5 * (y[0] + y[1]);
            double u_r = (s->mu * xi + s->kappa * y[1]) / (s->mu + s->kappa);
            double u_l = (s->mu * xi + s->kappa * y[0]) / (s->mu + s->kappa);
            if (up < u_l || up > u_r) {
                *ret = 0.0;
                return OQ_OK;
            }
            du = direction > 0 ? u_r - up : up - u_l;
        }
        if (du < best) {
            best = du;
        }
    }
    *ret = best;
    return OQ_OK;
}

/* advanceUniformly detail.h:2027-2050 (input_is_frame = false) */
static double advance_uniformly(oq_system* s, double du)
{
    double du_particles = du;
    double du_frame = du * (s->k_frame + s->mu) / s->k_frame;
    for (int64_t p = 0; p < s->N; ++p) {
        s->u[p] += du_particles;
    }
    s->u_frame += du_frame;
    updated_u(s);
    return du_frame;
}

/* eventDrivenStep detail.h:1933-1960 */
int oq_event_driven_step(oq_system* s, double eps, int kick, int direction, double* ret)
{
    double du;
    int rc;
    if (direction > 0 && !kick) {
        rc = oq_max_uniform_displacement(s, direction, &du);
        if (rc) {
            return rc;
        }
        if (du < 0.5 * eps) {
            *ret = 0.0;
            return OQ_OK;
        }
        *ret = advance_uniformly(s, du - 0.5 * eps);
        return OQ_OK;
    }
    if (direction > 0 && kick) {
        *ret = advance_uniformly(s, eps);
        return OQ_OK;
    }
    if (!kick) {
        rc = oq_max_uniform_displacement(s, direction, &du);
        if (rc) {
            return rc;
        }
        if (du < 0.5 * eps) {
            *ret = 0.0;
            return OQ_OK;
        }
        *ret = advance_uniformly(s, 0.5 * eps - du);
        return OQ_OK;
    }
    *ret = advance_uniformly(s, -eps);
    return OQ_OK;
}

/* trigger detail.h:1972-1977 (returns before updated_u); Cuspy::trigger :193-205 re-aligns first,
 * SemiSmooth::trigger :339-350 and Smooth::trigger :427-438 do not */
int oq_trigger(oq_system* s, int64_t p, double eps, int direction)
{
    if (p < 0 || p >= s->N) {
        return fail(s, OQ_ERR_INVALID, "particle index out of range");
    }
    if (s->pot == OQ_CUSPY) {
        align_all(s);
    }
    const double* y = s->data + p * s->n + s->cidx[p];
    if (direction > 0) {
        s->u[p] = y[1] + 0.5 * eps;
    }
    else {
        s->u[p] = y[0] - 0.5 * eps;
    }
    return OQ_OK;
}

/* advanceToFixedForce detail.h:1988-1995 */
int oq_advance_to_fixed_force(oq_system* s, double f_frame, int allow_plastic)
{
    int64_t N = s->N;
    int64_t* i_n = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    int64_t* cur = (int64_t*)malloc(sizeof(int64_t) * (size_t)N);
    gidx_all(s, i_n);
    double mean = reduce(s, s->f_frame, 0) / (double)N;
    advance_uniformly(s, (f_frame - mean) / s->mu);
    gidx_all(s, cur);
    int same = 1;
    for (int64_t p = 0; p < N; ++p) {
        if (cur[p] != i_n[p]) {
            same = 0;
        }
    }
    free(i_n);
    free(cur);
    if (!(allow_plastic || same)) {
        return fail(s, OQ_ERR_REQUIRE,
                    "assertion failed (allow_plastic || xt::all(xt::equal(m_chunk->index_at_align(), i_n)))");
    }
    return OQ_OK;
}

/* Canonical yield sequence of one particle p of a freshly constructed system, without building
 * the system: y_k for k in [k0, k0+count).  Used for spot checks at full problem sizes. */
int oq_sequence(uint64_t seed, int64_t p, int distribution, const double* parameters, int n_parameters, double offset,
                int64_t nchunk, int math_mode, int64_t k0, int64_t count, double* out)
{
    if (!dist_supported(distribution) || n_parameters > 4 || nchunk < 1) {
        return OQ_ERR_INVALID;
    }
    oq_system s;
    memset(&s, 0, sizeof(s));
    s.N = 1;
    s.n = nchunk;
    s.dist = distribution;
    s.npar = n_parameters;
    for (int i = 0; i < n_parameters; ++i) {
        s.par[i] = parameters[i];
    }
    s.offset = offset;
    s.math_mode = math_mode;
    uint64_t g0, inc;
    int restored = 0;
    int64_t kr = 0;
    uint64_t sr = 0;
    double yr = 0.0;
    pcg_seed(seed + (uint64_t)p, 0u, &g0, &inc);
    s.g0 = &g0;
    s.inc = &inc;
    s.restored = &restored;
    s.kr = &kr;
    s.sr = &sr;
    s.yr = &yr;
    seq_fill(&s, 0, k0, count, out);
    return OQ_OK;
}
