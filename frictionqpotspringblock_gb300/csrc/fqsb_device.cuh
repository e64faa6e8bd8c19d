/*
 * Device-side building blocks of the time-integration path (sm_103a, FP64).
 *
 * All floating-point arithmetic goes through __dadd_rn / __dmul_rn / ...
 * (FQ_* macros), so nvcc cannot contract it into fma and every kernel
 * reproduces the reference's operation order exactly
 * (include/FrictionQPotSpringBlock/detail.h:1539-1570 and the force functions
 * it calls).
 *
 * Disorder ("chunk"): per particle a window of W yield positions of the
 * particle's canonical yield sequence, plus the particle's current well
 * (yl, yr) and derived constants cached in one double4.  The canonical
 * sequence (one definition, independent of where the window sits):
 *     0 <= k < n0 : c_0 = d_0, c_k = c_{k-1} + d_k, y_k = c_k + offset
 *     k >= n0     : y_k = y_{k-1} + d_k
 *     k < 0       : y_k = y_{k+1} - d_{k+1}
 * with d_k the distribution transform of the k-th pcg32 output of the
 * particle's generator (initstate = seed + p, initseq = 0) and n0 = nchunk;
 * after chunk.restore(state, value, index) the sequence is redefined relative
 * to that anchor (y_index = value, forward by addition, backward by
 * subtraction).  This restates prrng's pcg32_tensor_cumsum (the reference's
 * Generator, Line1d.h:51-52) as used by the reference.
 */
#ifndef FQSB_DEVICE_CUH
#define FQSB_DEVICE_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "fq_math.h"
#include "fq_soft64.h"

namespace fqsb {

constexpr uint64_t PCG_MULT = 0x5851f42d4c957f2dULL;

enum : int { POT_CUSPY = 0, POT_SEMISMOOTH = 1, POT_SMOOTH = 2 };
enum : int {
    INTER_NONE = 0,
    INTER_LAPLACE1D = 1,
    INTER_LAPLACE2D = 2,
    INTER_QUARTIC1D = 3,     /* Quartic1d, detail.h:757-805 */
    INTER_QUARTICGRAD1D = 4, /* QuarticGradient1d, detail.h:616-653 */
    INTER_QUARTICGRAD2D = 5, /* QuarticGradient2d, detail.h:658-751 */
    INTER_LONGRANGE1D = 6    /* LongRange1d, detail.h:812-868 (all pairs on the ring) */
};

/* nearest neighbours on a periodic ring / on a periodic rows x cols grid */
__host__ __device__ constexpr bool inter_ring(int inter)
{
    return inter == INTER_LAPLACE1D || inter == INTER_QUARTIC1D || inter == INTER_QUARTICGRAD1D;
}
__host__ __device__ constexpr bool inter_grid(int inter)
{
    return inter == INTER_LAPLACE2D || inter == INTER_QUARTICGRAD2D;
}
enum : int {
    DIST_RANDOM = 0,
    DIST_DELTA = 1,
    DIST_EXPONENTIAL = 2,
    DIST_POWER = 3,
    DIST_GAMMA = 4,
    DIST_PARETO = 5,
    DIST_WEIBULL = 6,
    DIST_NORMAL = 7
};

/* termination codes of a stepping run (Ctl::done) */
enum : int { RUN_ACTIVE = 0, RUN_CONVERGED = 1, RUN_MAXITER = 2, RUN_EVENT = 3, RUN_TRUNCATED = 4 };
/* error codes (Ctl::error), equal to fqsb_status */
enum : int { DERR_NONE = 0, DERR_NAN = 1, DERR_WALK = 5 };

/* Upper bound on the draws one yield search may walk through; beyond it the search gives up
 * (flagging Ctl::walk_flag) instead of running for an unbounded time. */
constexpr int64_t MAX_WALK = int64_t(1) << 26;
/* run flags (Ctl::flags) */
enum : int { RF_RESID = 1, RF_ACT = 2, RF_FLOW = 4, RF_EVENT = 8, RF_TRUNCATE = 16,
             RF_SCHEDULE = 32, /* u_frame of step i is sched[i] (set before the step, as set_u_frame) */
             RF_RECORD = 64,   /* record each step's output u, v, a and well into rec_* [step][N] */
             RF_FFSUM = 128,   /* record each step's sum of f_frame (pairwise order) into rec_ffsum[step] */
             RF_NOINC = 256 }; /* the loop's iterations are not time steps: inc does not advance */

/* Control block of a stepping run; lives in device memory, written by the host before a run and
 * by the last CTA of every step. */
struct Ctl {
    /* run parameters */
    int64_t max_steps;
    double tol, tol2;
    int64_t niter_tol;
    int32_t flags;
    int32_t pad0;
    double vdt; /* v_frame * dt for flowSteps */
    int64_t A_truncate, S_truncate;
    /* run state */
    int32_t cur;
    int32_t done;
    int32_t error;
    uint32_t ticket;
    uint32_t ticket_redo;
    int32_t n_pending_cta; /* CTAs of this step with a particle whose chunk window must move */
    int32_t n_regen;       /* particles of this step whose chunk window must move */
    int32_t nx_stale;      /* the one-cluster kernel moved a window: next-window buffers to refresh */
    int64_t launch_steps;  /* steps done in the current graph launch */
    uint64_t launch_t0;    /* %globaltimer at the first step of the current graph launch */
    uint64_t budget_ns;    /* device time after which a graph launch yields back to the host */
    int64_t step;
    int64_t inc;
    double u_frame;
    /* StopList (GooseFEM::Iterate::StopList): ring + counters */
    int64_t sl_pos, sl_ge_tol, sl_ge_tol2, sl_asc;
    /* activity (detail.h:1768-1778, 1855-1866) */
    int64_t s_sum, a_count, s_n;
    int32_t init;
    int32_t nan_flag;
    int32_t walk_flag; /* a yield search exceeded MAX_WALK (absurd target): reported as an error */
    int32_t pad1;
    int64_t qs_first, qs_last;
    /* last residual (for diagnostics) */
    double last_residual;
    /* trajectory recording for the adjoint (RF_SCHEDULE / RF_RECORD / RF_FFSUM) */
    const double* sched;
    double *rec_u, *rec_v, *rec_a;
    double4_32a* rec_w;
    double* rec_ffsum;
};

/*
 * RandomNormalForcing (detail.h:881-1000): the pcg32 stream all draws come from, in particle order
 * (prrng's pcg32 m_state / m_inc), and the bookkeeping of one draw: the state before it (base) and
 * the ticket of its counting kernel.
 */
struct Thermal {
    uint64_t state;
    uint64_t inc;
    uint64_t base;  /* state before the current draw */
    int64_t total;  /* draws of the current draw */
    uint32_t ticket;
    uint32_t pad;
};

/* prrng pcg32(seed): the PCG seeding procedure on the default stream 0xda3e39cb94b95bdb */
constexpr uint64_t PCG_DEFAULT_STREAM = 0xda3e39cb94b95bdbULL;

/* LCG jump-ahead of a pcg32 stream with increment `inc` by delta steps (mod 2^64), Brown (1994),
 * "Random number generation with arbitrary strides". */
__host__ __device__ inline uint64_t pcg_advance_inc(uint64_t state, uint64_t delta, uint64_t inc)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = inc, acc_mult = 1ULL, acc_plus = 0ULL;
    while (delta > 0) {
        if (delta & 1ULL) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ULL) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    return acc_mult * state + acc_plus;
}

/* How a multiplication by a positive parameter c is carried out (all exact-equivalent to x * c). */
enum : int { SCALE_ONE = 0, SCALE_POW2 = 1, SCALE_GENERAL = 2 };

struct Scale {
    int mode; /* SCALE_* */
    int e;    /* c = 2^e when mode == SCALE_POW2 */
    double c;
};

struct DevSys {
    int64_t N, rows, cols;
    int pot, inter;
    double dt, hdt, hdt2, mu, kappa, k, k_frame, me, inv_m, m;
    /* Quartic1d: ia = a1, ib = a2; QuarticGradient: ia = k2, ib = k4, k4_4 = 0.25 k4 (1d),
     * qg_c2 = k2 + k4 / 3 and qg_k23 = 2 (k4 / 3) (2d), each rounded as the reference forms them */
    double ia, ib, k4_4, qg_c2, qg_k23;
    const double* lr_pref; /* LongRange1d: k / d^(alpha + 1) by ring distance d (0 at d = 0), host std::pow */
    int64_t lr_m;          /* LongRange1d: ring distances above lr_m wrap to N - d */
    Scale s_mu, s_k, s_kf, s_im; /* mu, k_interactions, k_frame, 1/m */
    /* chunk */
    int64_t W, n0;
    int dist, npar;
    double par[4];
    double offset;
    const double* offp;
    uint64_t seed;
    const uint64_t* pseed; /* per-particle pcg32 initstate (batched realisations), or NULL: seed + p */
    int64_t buffer, margin, min_margin;
    double* data;
    int64_t* start;
    int32_t* cidx;
    int64_t* gidx;
    double4_32a* wc;
    double* acc_end;
    double* nx;      /* next-window buffer [N, W] of small systems (next_window_ready), or NULL */
    int64_t* nx_end; /* window end the buffer of particle p follows */
    uint8_t* anc_kind;
    int64_t* anc_k;
    uint64_t* anc_state;
    double* anc_val;
    /* state, double buffered */
    double* u[2];
    double* v[2];
    double* a[2];
    /* run control */
    Ctl* ctl;
    double* ring;
    double2* partials;
    int64_t* i_n;
    double2* sq2;
    int64_t npartials;
    int32_t* cta_pending; /* per CTA of the step grid */
    int32_t* regen_list;  /* particles whose chunk window must move (capacity N) */
    unsigned long long h_while; /* cudaGraphConditionalHandle of the run loop */
    unsigned long long h_if;    /* cudaGraphConditionalHandle of the regeneration branch */
    int in_graph;               /* 0: kernels launched one by one by the host (no conditional handles) */
    /* RandomNormalForcing (f_th == NULL: none) */
    double* f_th;       /* f_thermal [N] */
    int64_t* th_next;   /* next increment at which particle p redraws */
    const int64_t* th_dinc;
    int64_t* th_cnt;    /* per 1024-particle tile: draws, then their exclusive prefix */
    int32_t* th_list;   /* the drawing particles in flat order (capacity N) */
    Thermal* th;
    double th_mean, th_sc; /* mean and stddev * sqrt(2) (rounded as the reference's normal transform) */
};

/* ------------------------------------------------------------ pcg32 */

__device__ __forceinline__ uint32_t pcg_output(uint64_t old)
{
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return __funnelshift_r(xs, xs, rot);
}

__device__ __forceinline__ uint64_t pcg_step(uint64_t s)
{
    return s * PCG_MULT + 1ULL; /* initseq = 0 => inc = 1 */
}

/* pcg32_srandom_r(initstate, initseq = 0) */
__device__ __forceinline__ uint64_t pcg_seed(uint64_t initstate)
{
    uint64_t s = pcg_step(0ULL);
    s += initstate;
    return pcg_step(s);
}

/* LCG jump-ahead by delta (mod 2^64), Brown (1994) */
static __device__ __noinline__ uint64_t pcg_advance(uint64_t state, uint64_t delta)
{
    uint64_t cur_mult = PCG_MULT, cur_plus = 1ULL, acc_mult = 1ULL, acc_plus = 0ULL;
    while (delta > 0) {
        if (delta & 1ULL) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1ULL) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    return acc_mult * state + acc_plus;
}

__device__ __forceinline__ double par_or(const DevSys& s, int i, double def)
{
    return i < s.npar ? s.par[i] : def;
}

/* prrng distribution transform of one draw; same expressions and order as the oracle */
__device__ __forceinline__ double dev_transform_inl(const DevSys& s, uint32_t r32)
{
    double r = FQ_MUL((double)r32, 0x1p-32);
    switch (s.dist) {
        case DIST_RANDOM:
            return FQ_ADD(FQ_MUL(r, par_or(s, 0, 1.0)), par_or(s, 1, 0.0));
        case DIST_DELTA:
            return FQ_ADD(par_or(s, 0, 1.0), par_or(s, 1, 0.0));
        case DIST_EXPONENTIAL:
            return FQ_ADD(FQ_MUL(-fq_log(FQ_SUB(1.0, r)), par_or(s, 0, 1.0)), par_or(s, 1, 0.0));
        case DIST_POWER:
            return FQ_ADD(fq_pow(r, FQ_DIV(1.0, par_or(s, 0, 1.0))), par_or(s, 1, 0.0));
        case DIST_PARETO:
            return FQ_ADD(FQ_DIV(par_or(s, 1, 1.0), fq_pow(FQ_SUB(1.0, r), FQ_DIV(1.0, par_or(s, 0, 1.0)))),
                          par_or(s, 2, 0.0));
        case DIST_WEIBULL:
            return FQ_ADD(FQ_MUL(par_or(s, 1, 1.0), fq_pow(-fq_log(FQ_SUB(1.0, r)), FQ_DIV(1.0, par_or(s, 0, 1.0)))),
                          par_or(s, 2, 0.0));
        default:
            return __longlong_as_double(0x7ff8000000000000LL);
    }
}

/* out of line where it is called in a loop (keeps the callers' registers low) */
static __device__ __noinline__ double dev_transform(const DevSys& s, uint32_t r32)
{
    return dev_transform_inl(s, r32);
}

__device__ __forceinline__ double dev_draw(const DevSys& s, uint64_t st)
{
    return dev_transform(s, s.dist == DIST_DELTA ? 0u : pcg_output(st));
}

__device__ __forceinline__ double off_of(const DevSys& s, int64_t p)
{
    return s.offp ? s.offp[p] : s.offset;
}

/* origin of the particle's sequence: index, and pcg32 state whose output is d_origin */
__device__ __forceinline__ void seq_origin(const DevSys& s, int64_t p, int& kind, int64_t& k0, uint64_t& st0)
{
    kind = s.anc_kind[p];
    if (kind) {
        k0 = s.anc_k[p];
        st0 = s.anc_state[p];
    }
    else {
        k0 = 0;
        st0 = pcg_seed(s.pseed ? s.pseed[p] : s.seed + (uint64_t)p);
    }
}

/*
 * Canonical y_k for k in [k0, k0+cnt) written to out[0..cnt), replayed from the particle's origin.
 * Also returns, if acc_last != NULL, the running accumulator at index k0+cnt-1 (c_k inside the
 * initial region 0 <= k < n0, else y_k), which lets a later forward extension continue exactly.
 */
static __device__ __noinline__ void seq_fill(const DevSys& s, int64_t p, int64_t k0, int64_t cnt, double* out,
                                      double* acc_last)
{
    int kind;
    int64_t ko;
    uint64_t sto;
    seq_origin(s, p, kind, ko, sto);
    int64_t k1 = k0 + cnt;
    double acc_out = 0.0;
    if (kind) {
        double yr = s.anc_val[p];
        if (k1 > ko) {
            double y = yr;
            uint64_t st = sto;
            if (ko >= k0) {
                out[ko - k0] = y;
            }
            for (int64_t k = ko + 1; k < k1; ++k) {
                st = pcg_step(st);
                y = FQ_ADD(y, dev_draw(s, st));
                if (k >= k0) {
                    out[k - k0] = y;
                }
            }
            if (k1 - 1 >= ko) {
                acc_out = y;
            }
        }
        if (k0 < ko) {
            double y = yr;
            uint64_t st = sto;
            for (int64_t k = ko - 1; k >= k0; --k) {
                y = FQ_SUB(y, dev_draw(s, st));
                if (k < k1) {
                    out[k - k0] = y;
                    if (k == k1 - 1) {
                        acc_out = y;
                    }
                }
                st = pcg_advance(st, ~0ULL);
            }
        }
    }
    else {
        int64_t n0 = s.n0;
        double o = off_of(s, p);
        if (k1 > 0) {
            uint64_t st = sto;
            double c = 0.0, y = 0.0;
            for (int64_t k = 0; k < k1; ++k) {
                double d = dev_draw(s, st);
                if (k == 0) {
                    c = d;
                    y = FQ_ADD(c, o);
                }
                else if (k < n0) {
                    c = FQ_ADD(c, d);
                    y = FQ_ADD(c, o);
                }
                else {
                    y = FQ_ADD(y, d);
                }
                if (k >= k0) {
                    out[k - k0] = y;
                }
                st = pcg_step(st);
            }
            acc_out = (k1 - 1 < n0) ? c : y;
        }
        if (k0 < 0) {
            double y = FQ_ADD(dev_draw(s, sto), o);
            uint64_t st = sto;
            for (int64_t k = -1; k >= k0; --k) {
                y = FQ_SUB(y, dev_draw(s, st));
                if (k < k1) {
                    out[k - k0] = y;
                    if (k == k1 - 1) {
                        acc_out = y;
                    }
                }
                st = pcg_advance(st, ~0ULL);
            }
        }
    }
    if (acc_last) {
        *acc_last = acc_out;
    }
}

/* Forward walker over the canonical sequence, valid at indices >= the origin. */
struct Walker {
    int64_t k;   /* index of the last produced value */
    double acc;  /* accumulator at k (c_k in the initial region, else y_k) */
    double y;    /* y_k */
    uint64_t st; /* pcg32 state whose output is d_{k+1} */
    int kind;
    int64_t n0;
    double o;
};

__device__ __forceinline__ void walker_next(const DevSys& s, Walker& w)
{
    double d = dev_draw(s, w.st);
    w.st = pcg_step(w.st);
    int64_t k = w.k + 1;
    if (w.kind) {
        w.acc = FQ_ADD(w.acc, d);
        w.y = w.acc;
    }
    else if (k < w.n0) {
        w.acc = FQ_ADD(w.acc, d);
        w.y = FQ_ADD(w.acc, w.o);
    }
    else if (k == w.n0) {
        w.y = FQ_ADD(FQ_ADD(w.acc, w.o), d);
        w.acc = w.y;
    }
    else {
        w.acc = FQ_ADD(w.acc, d);
        w.y = w.acc;
    }
    w.k = k;
}

/* Refresh the cached well of particle p from its chunk row at chunk index li. */
__device__ __forceinline__ double4_32a make_wc(const DevSys& s, double yl, double yr)
{
    double4_32a w;
    w.x = yl;
    w.y = yr;
    if (s.pot == POT_SEMISMOOTH) {
        double xi = FQ_MUL(0.5, FQ_ADD(yl, yr));
        double den = FQ_ADD(s.mu, s.kappa);
        w.z = FQ_DIV(FQ_ADD(FQ_MUL(s.mu, xi), FQ_MUL(s.kappa, yl)), den); /* u_l */
        w.w = FQ_DIV(FQ_ADD(FQ_MUL(s.mu, xi), FQ_MUL(s.kappa, yr)), den); /* u_r */
    }
    else {
        w.z = FQ_MUL(0.5, FQ_ADD(yl, yr)); /* well centre */
        w.w = FQ_MUL(0.5, FQ_SUB(yr, yl)); /* half width (Smooth) */
    }
    return w;
}

/*
 * prrng align for particle p at target u: find i with y[i] <= u < y[i+1]; when i leaves
 * [min_margin, W - buffer) move the window so that the target sits at chunk index `margin`.
 * Updates start, cidx, gidx, wc, acc_end of the particle.  Returns false for a non-finite u
 * (the index is then kept; the NaN is reported by the step's NaN check).
 */
static __device__ __noinline__ bool dev_align(const DevSys& s, int64_t p, double u)
{
    if (!(u == u) || fabs(u) == __longlong_as_double(0x7ff0000000000000LL)) {
        return false;
    }
    const int64_t W = s.W;
    double* y = s.data + p * W;
    int64_t start = s.start[p];
    int64_t li = s.cidx[p];
    int64_t gi;
    int kind;
    int64_t ko;
    uint64_t sto;
    seq_origin(s, p, kind, ko, sto);
    if (y[0] <= u && u < y[W - 1]) {
        if (y[li] <= u) {
            while (li + 1 < W && y[li + 1] <= u) {
                ++li;
            }
        }
        else {
            while (li > 0 && y[li] > u) {
                --li;
            }
        }
        if (li >= s.min_margin && li < W - s.buffer) {
            s.cidx[p] = (int32_t)li;
            s.gidx[p] = start + li;
            s.wc[p] = make_wc(s, y[li], y[li + 1]);
            return true;
        }
        gi = start + li;
    }
    else if (u >= y[W - 1]) {
        gi = -1; /* found below */
    }
    else {
        gi = -2;
    }

    int64_t end = start + W - 1;
    bool fast = end >= ko; /* the forward walker is exact from the window end */
    if (gi == -1) {
        if (fast) {
            Walker w;
            w.k = end;
            w.acc = s.acc_end[p];
            w.y = y[W - 1];
            w.st = pcg_advance(sto, (uint64_t)(end + 1 - ko));
            w.kind = kind;
            w.n0 = s.n0;
            w.o = off_of(s, p);
            for (int64_t it = 0;; ++it) {
                if (it >= MAX_WALK) {
                    atomicOr(&s.ctl->walk_flag, 1);
                    return false;
                }
                walker_next(s, w);
                if (w.y > u) {
                    gi = w.k - 1;
                    break;
                }
            }
        }
        else {
            /* window lies left of the origin: scan forward block by block by replay */
            int64_t k = end;
            for (int64_t it = 0;; ++it) {
                if (it * 64 >= MAX_WALK) {
                    atomicOr(&s.ctl->walk_flag, 1);
                    return false;
                }
                double blk[64];
                seq_fill(s, p, k + 1, 64, blk, nullptr);
                int64_t j = 0;
                while (j < 64 && blk[j] <= u) {
                    ++j;
                }
                if (j < 64) {
                    gi = k + j;
                    break;
                }
                k += 64;
            }
        }
    }
    else if (gi == -2) {
        int64_t k = start; /* y_k > u */
        for (int64_t it = 0;; ++it) {
            if (it * 64 >= MAX_WALK) {
                atomicOr(&s.ctl->walk_flag, 1);
                return false;
            }
            double blk[64];
            seq_fill(s, p, k - 64, 64, blk, nullptr);
            int64_t j = 63;
            while (j >= 0 && blk[j] > u) {
                --j;
            }
            if (j >= 0) {
                gi = k - 64 + j;
                break;
            }
            k -= 64;
        }
    }

    int64_t ns = gi - s.margin;
    double acc = 0.0;
    if (ns > start && fast) {
        /* forward move: keep the overlap, extend by the walker from the old window end */
        int64_t keep = end + 1 - ns; /* values of the old window that stay (may be <= 0) */
        if (keep > 0) {
            for (int64_t j = 0; j < keep; ++j) {
                y[j] = y[j + (ns - start)];
            }
        }
        Walker w;
        w.k = end;
        w.acc = s.acc_end[p];
        w.y = 0.0;
        w.st = pcg_advance(sto, (uint64_t)(end + 1 - ko));
        w.kind = kind;
        w.n0 = s.n0;
        w.o = off_of(s, p);
        int64_t first = keep > 0 ? keep : 0;
        while (w.k < ns + first - 1) {
            walker_next(s, w);
        }
        for (int64_t j = first; j < W; ++j) {
            walker_next(s, w);
            y[j] = w.y;
        }
        acc = w.acc;
    }
    else {
        seq_fill(s, p, ns, W, y, &acc);
    }
    s.start[p] = ns;
    s.acc_end[p] = acc;
    li = s.margin;
    s.cidx[p] = (int32_t)li;
    s.gidx[p] = ns + li;
    s.wc[p] = make_wc(s, y[li], y[li + 1]);
    return true;
}

/*
 * Cooperative forward window move.  A move costs W - keep draws, each a distribution transform of
 * some hundred dependent fp64 operations (the portable double-double log of the Weibull / exponential
 * transforms); one thread doing them alone stalls its CTA (and, in the one-cluster kernel, the whole
 * cluster) for ~1 ms.  The draws are independent given their pcg32 states, so the threads of a CTA
 * share them; only the running sum, one addition per value, stays with the particle's own thread and
 * runs in the sequence's order -- the values are the ones dev_align writes, bit for bit.
 *
 * Applies when u lies inside the window but its index has passed the upper margin (the usual way a
 * particle leaves its window in a dynamic run) and the forward walker is exact from the window end;
 * every other move goes through dev_align.
 */
struct FwdMove {
    int64_t p, ns, keep;
    uint64_t st_first; /* pcg32 state whose output is the draw of index old end + 1 */
    int32_t next;      /* the new slots come from the next-window buffer (next_window_ready) */
    int32_t pad;
};

/* Forward shift of a window's kept values, y[j] = y[j + sh] for j < keep, in blocks of 16 loads
 * ahead of their stores (a later block reads only slots above the ones written so far). */
static __device__ __noinline__ void window_shift(double* y, int64_t keep, int64_t sh)
{
    constexpr int B = 16;
    for (int64_t j0 = 0; j0 < keep; j0 += B) {
        double t[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            t[i] = j0 + i < keep ? y[j0 + i + sh] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (j0 + i < keep) {
                y[j0 + i] = t[i];
            }
        }
    }
}

/* Plans the move of particle p to target u; on success also copies the kept values down. */
__device__ __forceinline__ bool fwd_move_plan(const DevSys& s, int64_t p, double u, FwdMove& m)
{
    if (!(u == u)) {
        return false;
    }
    const int64_t W = s.W;
    double* y = s.data + p * W;
    if (!(y[0] <= u && u < y[W - 1])) {
        return false;
    }
    int64_t li = s.cidx[p];
    if (y[li] <= u) {
        while (li + 1 < W && y[li + 1] <= u) {
            ++li;
        }
    }
    else {
        while (li > 0 && y[li] > u) {
            --li;
        }
    }
    if (li < W - s.buffer) {
        return false; /* inside the margins, or a move down */
    }
    const int64_t start = s.start[p];
    const int64_t ns = start + li - s.margin;
    const int64_t end = start + W - 1;
    const int64_t keep = end + 1 - ns;
    int kind;
    int64_t ko;
    uint64_t sto;
    seq_origin(s, p, kind, ko, sto);
    if (ns <= start || keep <= 0 || end < ko) {
        return false;
    }
    window_shift(y, keep, ns - start);
    m.p = p;
    m.ns = ns;
    m.keep = keep;
    m.st_first = pcg_advance(sto, (uint64_t)(end + 1 - ko));
    m.next = 0;
    return true;
}

/* Draws of cnt consecutive sequence indices into dst[0..cnt), the first from pcg32 state st_first:
 * thread `lane` of `nlanes` writes slots lane, lane + nlanes, ... (one jump-ahead, then strides of
 * nlanes steps: the stride map x -> a x + c with c = advance(0, nlanes), a = advance(1, nlanes) - c). */
static __device__ __noinline__ void seq_draws(const DevSys& s, double* dst, int64_t cnt, uint64_t st_first, int lane,
                                              int nlanes, uint64_t sa, uint64_t sc)
{
    /* two draws per iteration (slots j and j + nlanes), inlined, so that their long dependency chains
     * overlap; stride 2 nlanes: x -> sa2 x + sc2 */
    const uint64_t sa2 = sa * sa, sc2 = sa * sc + sc;
    uint64_t st0 = pcg_advance(st_first, (uint64_t)lane);
    uint64_t st1 = sa * st0 + sc;
    const bool delta = s.dist == DIST_DELTA;
    for (int64_t j = lane; j < cnt; j += 2 * (int64_t)nlanes) {
        const double d0 = dev_transform_inl(s, delta ? 0u : pcg_output(st0));
        const double d1 = dev_transform_inl(s, delta ? 0u : pcg_output(st1));
        dst[j] = d0;
        if (j + nlanes < cnt) {
            dst[j + nlanes] = d1;
        }
        st0 = sa2 * st0 + sc2;
        st1 = sa2 * st1 + sc2;
    }
}

/* Draws of one planned move: window slots keep .. W - 1 */
__device__ __forceinline__ void fwd_move_draws(const DevSys& s, const FwdMove& m, int lane, int nlanes, uint64_t sa,
                                               uint64_t sc)
{
    seq_draws(s, s.data + m.p * s.W + m.keep, s.W - m.keep, m.st_first, lane, nlanes, sa, sc);
}

/* The running sum of one planned move over its drawn slots, in the sequence's order (walker_next's
 * rules), then the particle's window bookkeeping as dev_align leaves it. */
__device__ __forceinline__ void fwd_move_sum(const DevSys& s, const FwdMove& m)
{
    const int64_t W = s.W, p = m.p;
    double* y = s.data + p * W;
    int kind;
    int64_t ko;
    uint64_t sto;
    seq_origin(s, p, kind, ko, sto);
    const int64_t n0 = s.n0;
    const double o = off_of(s, p);
    double acc = s.acc_end[p];
    /* the draws are read in blocks of 16 independent loads, so that the chain of additions, not the
     * memory latency, sets the pace */
    constexpr int B = 16;
    for (int64_t j0 = m.keep; j0 < W; j0 += B) {
        double d[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            d[i] = j0 + i < W ? __ldcg(y + j0 + i) : 0.0;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            const int64_t j = j0 + i;
            if (j >= W) {
                break;
            }
            const int64_t k = m.ns + j;
            double yk;
            if (kind) {
                acc = FQ_ADD(acc, d[i]);
                yk = acc;
            }
            else if (k < n0) {
                acc = FQ_ADD(acc, d[i]);
                yk = FQ_ADD(acc, o);
            }
            else if (k == n0) {
                yk = FQ_ADD(FQ_ADD(acc, o), d[i]);
                acc = yk;
            }
            else {
                acc = FQ_ADD(acc, d[i]);
                yk = acc;
            }
            d[i] = yk;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (j0 + i < W) {
                y[j0 + i] = d[i];
            }
        }
    }
    s.start[p] = m.ns;
    s.acc_end[p] = acc;
    const int64_t li = s.margin;
    s.cidx[p] = (int32_t)li;
    s.gidx[p] = m.ns + li;
    s.wc[p] = make_wc(s, y[li], y[li + 1]);
}

/*
 * Next-window buffer of the one-cluster kernel of small systems.  nx[p * W + j] holds y_k of the
 * W sequence indices k = end + 1 + j after the window end `end` = nx_end[p], computed ahead of the
 * run (k_next_window) by the rules of fwd_move_sum, so that a forward move inside the run copies its
 * new slots instead of drawing them: a move then costs a copy, not W - keep distribution transforms
 * on one SM while the whole cluster waits.  Held for indices past the initial region only (there the
 * accumulator equals y_k, which fixes acc_end after the move); other windows keep the drawn moves.
 */
__device__ __forceinline__ bool next_window_ready(const DevSys& s, int64_t p)
{
    return s.nx != nullptr && s.nx_end[p] == s.start[p] + s.W - 1;
}

/* Whether the buffer can hold the indices after window end `end` of particle p; also the origin */
__device__ __forceinline__ bool next_window_applies(const DevSys& s, int64_t p, int64_t end, int& kind, int64_t& ko,
                                                    uint64_t& sto)
{
    seq_origin(s, p, kind, ko, sto);
    return end >= ko && (kind != 0 || end + 1 >= s.n0);
}

/* The running sum over drawn slots nx[p * W ...] after window end `end`, in place (one thread) */
static __device__ __noinline__ void next_window_sum(const DevSys& s, int64_t p, int64_t end, int kind)
{
    const int64_t W = s.W, n0 = s.n0;
    double* y = s.nx + p * W;
    const double o = off_of(s, p);
    double acc = s.acc_end[p];
    constexpr int B = 16;
    for (int64_t j0 = 0; j0 < W; j0 += B) {
        double d[B];
#pragma unroll
        for (int i = 0; i < B; ++i) {
            d[i] = j0 + i < W ? __ldcg(y + j0 + i) : 0.0;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (j0 + i >= W) {
                break;
            }
            if (kind == 0 && end + 1 + j0 + i == n0) {
                acc = FQ_ADD(FQ_ADD(acc, o), d[i]);
            }
            else {
                acc = FQ_ADD(acc, d[i]);
            }
            d[i] = acc;
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
            if (j0 + i < W) {
                y[j0 + i] = d[i];
            }
        }
    }
}

/* A planned move whose new slots are in the next-window buffer: thread `lane` of `nlanes` copies
 * slots keep + lane, keep + lane + nlanes, ... */
__device__ __forceinline__ void fwd_move_copy(const DevSys& s, const FwdMove& m, int lane, int nlanes)
{
    const int64_t W = s.W;
    double* y = s.data + m.p * W;
    const double* x = s.nx + m.p * W;
    for (int64_t j = m.keep + lane; j < W; j += nlanes) {
        y[j] = __ldcg(x + (j - m.keep));
    }
}

/* The window bookkeeping of a copied move, as fwd_move_sum leaves it */
__device__ __forceinline__ void fwd_move_finish(const DevSys& s, const FwdMove& m)
{
    const int64_t W = s.W, p = m.p;
    double* y = s.data + p * W;
    s.start[p] = m.ns;
    s.acc_end[p] = __ldcg(s.nx + p * W + (W - 1 - m.keep));
    const int64_t li = s.margin;
    s.cidx[p] = (int32_t)li;
    s.gidx[p] = m.ns + li;
    s.wc[p] = make_wc(s, y[li], y[li + 1]);
}

/* ------------------------------------------- exact integer-pipe helpers */

/* Order-preserving integer key of a double: key(a) < key(b) <=> a < b for all non-NaN a, b, with
 * key(-0) == key(+0).  Positive NaNs sort above +inf and negative NaNs below -inf, so a NaN position
 * never passes the well test (as the fp64 comparison). */
__device__ __forceinline__ long long dkey(double x)
{
    long long b = __double_as_longlong(x);
    long long sgn = b >> 63;
    return (b ^ (sgn & 0x7fffffffffffffffLL)) - sgn;
}

/* yl <= u < yr, evaluated on the integer pipe (identical result to the fp64 comparisons). */
__device__ __forceinline__ bool in_well(double yl, double yr, double u)
{
    long long k = dkey(u);
    return dkey(yl) <= k && k < dkey(yr);
}

/*
 * Per-operation choice of unit.  Bit i of SOFT set: operation site i of the particle update runs on
 * the integer pipes (fq_soft64.h, bit-identical to the hardware instruction); clear: on the fp64
 * pipe.  Sites: 0 dt*v, 1 hdt2*a, 2 u+dt*v, 3 +hdt2*a (position); 4 u_frame-u', 5 c-u' (Cuspy),
 * 6 f_frame+f_pot, 7 uL-2u', 8 +uR, 9 +f_int (forces); 10 dt*a0, 11 v0+dt*a0, 12 -eta*v, 13 s+(-eta*v)
 * (first velocity update); 14 a0+a, 15 hdt*(a0+a), 16 v0+hdt*(..), 17 -eta*v, 18 s+(-eta*v) (second)
 * and 19..23 the same for the third.
 */
#define S_ADD(bit, a, b) (((SOFT >> (bit)) & 1u) ? fq_sadd((a), (b)) : FQ_ADD((a), (b)))
#define S_SUB(bit, a, b) (((SOFT >> (bit)) & 1u) ? fq_ssub((a), (b)) : FQ_SUB((a), (b)))
#define S_MUL(bit, a, b) (((SOFT >> (bit)) & 1u) ? fq_smul((a), (b)) : FQ_MUL((a), (b)))

/*
 * The split the step kernels use: all eight multiplications and the two additions of the position
 * update on the integer pipes, the other fourteen additions on the fp64 pipe.  Measured on the
 * N = 2^22 flow workload against other splits (all multiplications only; also the velocity or the
 * force additions): 20.2 G particle-steps/s against 19.2-20.2 for the others and 14.8 with none.
 */
constexpr unsigned STEP_SOFT = (1u << 0) | (1u << 1) | (1u << 2) | (1u << 3) | (1u << 10) | (1u << 12) | (1u << 15) |
                               (1u << 17) | (1u << 20) | (1u << 22);

/* fp64 add / mul for work inside a run-time branch (residual and frame-force sums): volatile, so the
 * compiler cannot execute them speculatively before the branch, as it does with the plain forms. */
__device__ __forceinline__ double add_nospec(double a, double b)
{
    double r;
    asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
__device__ __forceinline__ double mul_nospec(double a, double b)
{
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}

__device__ __forceinline__ bool is_nan_bits(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

/* x * 2^e for a positive power of two: an exponent add when the result stays a normal number, exact
 * like the fp64 multiplication; zeros pass through; other cases use the fp64 multiply. */
__device__ __forceinline__ double scale_pow2(double x, int e, double c)
{
    long long b = __double_as_longlong(x);
    int ex = (int)((b >> 52) & 0x7ff);
    int ne = ex + e;
    if (ex != 0 && ex != 0x7ff && ne >= 1 && ne <= 0x7fe) {
        return __longlong_as_double(b + ((long long)e << 52));
    }
    if ((b & 0x7fffffffffffffffLL) == 0) {
        return x;
    }
    return FQ_MUL(x, c);
}

/* x * c with c described by sc (c > 0 for the power-of-two forms). */
__device__ __forceinline__ double scale(double x, const Scale& sc)
{
    if (sc.mode == SCALE_ONE) {
        return x;
    }
    if (sc.mode == SCALE_POW2) {
        return scale_pow2(x, sc.e, sc.c);
    }
    return FQ_MUL(x, sc.c);
}

/* Potential force, Cuspy detail.h:139-170 / SemiSmooth :236-277 / Smooth :379-409. */
template <int POT, unsigned SOFT = 0u>
__device__ __forceinline__ double pot_force(const DevSys& s, const double4_32a& w, double up)
{
    if (POT == POT_CUSPY) {
        return scale((SOFT >> 5) & 1u ? fq_ssub(w.z, up) : FQ_SUB(w.z, up), s.s_mu);
    }
    else if (POT == POT_SEMISMOOTH) {
        if (up < w.z) {
            return FQ_MUL(s.kappa, FQ_SUB(up, w.x));
        }
        else if (up <= w.w) {
            return FQ_MUL(s.mu, FQ_SUB(FQ_MUL(0.5, FQ_ADD(w.x, w.y)), up));
        }
        return FQ_MUL(s.kappa, FQ_SUB(up, w.y));
    }
    else {
        const double pi = 3.14159265358979323846;
        double arg = FQ_DIV(FQ_MUL(pi, FQ_SUB(up, w.z)), w.w);
        return FQ_MUL(FQ_DIV(FQ_MUL(-s.mu, w.w), pi), fq_sin(arg));
    }
}

/* ------------------------------------------------ interactions */

/*
 * f_interactions of a particle on a ring from its own and its two neighbours' positions.
 * Laplace1d detail.h:474-487 ((uL - 2u) + uR, then times k); Quartic1d :781-803
 * (a1 ((uL - 2u) + uR) + a2 ((dup dup) dup + (dun dun) dun), dup = uR - u, dun = uL - u);
 * QuarticGradient1d :636-650 (((uL - 2u) + uR) (k2 + (k4/4 du) du), du = uR - uL).
 * SOFT selects the integer-pipe forms of the Laplace1d operations (sites 7, 8).
 */
template <int INTER, unsigned SOFT = 0u>
__device__ __forceinline__ double ring_force(const DevSys& s, double uL, double u, double uR)
{
    if (INTER == INTER_LAPLACE1D) {
        return scale(S_ADD(8, S_SUB(7, uL, scale_pow2(u, 1, 2.0)), uR), s.s_k);
    }
    const double lap = FQ_ADD(FQ_SUB(uL, scale_pow2(u, 1, 2.0)), uR);
    if (INTER == INTER_QUARTIC1D) {
        const double dup = FQ_SUB(uR, u), dun = FQ_SUB(uL, u);
        return FQ_ADD(FQ_MUL(s.ia, lap),
                      FQ_MUL(s.ib, FQ_ADD(FQ_MUL(FQ_MUL(dup, dup), dup), FQ_MUL(FQ_MUL(dun, dun), dun))));
    }
    const double du = FQ_SUB(uR, uL);
    return FQ_MUL(lap, FQ_ADD(s.ia, FQ_MUL(FQ_MUL(s.k4_4, du), du)));
}

/*
 * QuarticGradient2d (detail.h:677-750) of cell (i, j) from its 3 x 3 neighbourhood: uip = u(i+1, j),
 * uim = u(i-1, j), ujp = u(i, j+1), ujm = u(i, j-1), upp = u(i+1, j+1), upm = u(i+1, j-1),
 * ump = u(i-1, j+1), umm = u(i-1, j-1), in the reference's order of operations.
 */
__device__ __forceinline__ double qg2d_force(const DevSys& s, double u, double uip, double uim, double ujp, double ujm,
                                             double upp, double upm, double ump, double umm)
{
    const double u2 = scale_pow2(u, 1, 2.0);
    const double l = FQ_SUB(FQ_ADD(FQ_ADD(FQ_ADD(uip, uim), ujp), ujm), scale_pow2(u, 2, 4.0));
    const double dudx = FQ_MUL(0.5, FQ_SUB(uip, uim));
    const double dudy = FQ_MUL(0.5, FQ_SUB(ujp, ujm));
    const double d2udxdy = FQ_MUL(0.25, FQ_ADD(FQ_SUB(FQ_SUB(upp, upm), ump), umm));
    const double d2udx2 = FQ_ADD(FQ_SUB(uip, u2), uim);
    const double d2udy2 = FQ_ADD(FQ_SUB(ujp, u2), ujm);
    const double t = FQ_ADD(FQ_ADD(FQ_MUL(FQ_MUL(dudx, dudx), d2udx2), FQ_MUL(FQ_MUL(dudy, dudy), d2udy2)),
                            FQ_MUL(FQ_MUL(FQ_MUL(2.0, dudx), dudy), d2udxdy));
    return FQ_ADD(FQ_MUL(l, s.qg_c2), FQ_MUL(s.qg_k23, t));
}

/* f_interactions of particle p from the positions u (any interaction type; no shared memory). */
__device__ __forceinline__ double inter_force_at(const DevSys& s, const double* u, int64_t p)
{
    if (inter_ring(s.inter)) {
        const int64_t N = s.N;
        const double uL = u[p == 0 ? N - 1 : p - 1], uR = u[p == N - 1 ? 0 : p + 1];
        switch (s.inter) {
            case INTER_LAPLACE1D: return ring_force<INTER_LAPLACE1D>(s, uL, u[p], uR);
            case INTER_QUARTIC1D: return ring_force<INTER_QUARTIC1D>(s, uL, u[p], uR);
            default: return ring_force<INTER_QUARTICGRAD1D>(s, uL, u[p], uR);
        }
    }
    if (s.inter == INTER_LONGRANGE1D) {
        /* LongRange1d::force detail.h:844-866: sequential sum over i != p in index order */
        const int64_t N = s.N;
        const double up = u[p];
        double fp = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            if (i == p) {
                continue;
            }
            int64_t d = i > p ? i - p : p - i;
            if (d > s.lr_m) {
                d = N - d;
            }
            fp = FQ_ADD(fp, FQ_MUL(FQ_SUB(u[i], up), s.lr_pref[d]));
        }
        return fp;
    }
    if (inter_grid(s.inter)) {
        const int64_t R = s.rows, C = s.cols, i = p / C, j = p % C;
        const int64_t im = (i + R - 1) % R, ip = (i + 1) % R, jm = (j + C - 1) % C, jp = (j + 1) % C;
        if (s.inter == INTER_LAPLACE2D) {
            /* Laplace2d detail.h:545-583: (((u(i-1,j) + u(i+1,j)) + u(i,j-1)) + u(i,j+1)) - 4 u, then times k */
            return scale(FQ_SUB(FQ_ADD(FQ_ADD(FQ_ADD(u[im * C + j], u[ip * C + j]), u[i * C + jm]), u[i * C + jp]),
                                scale_pow2(u[p], 2, 4.0)),
                         s.s_k);
        }
        return qg2d_force(s, u[p], u[ip * C + j], u[im * C + j], u[i * C + jp], u[i * C + jm], u[ip * C + jp],
                          u[ip * C + jm], u[im * C + jp], u[im * C + jm]);
    }
    return 0.0;
}

/* ------------------------------------------------ canonical reductions */

/* Sum over the 32 lanes in the fixed pairwise order (lane i with i+1, then pairs of pairs, ...), the
 * result in lane 0.  At level m only the lanes that start a pair of width 2m add (the others' values
 * are no longer needed); the add is non-speculatable so that the idle lanes do not issue it (the fp64
 * pipe's cost follows the active lanes). */
__device__ __forceinline__ double warp_tree(double x)
{
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        double y = __shfl_down_sync(0xffffffffu, x, m);
        if ((threadIdx.x & (2 * m - 1)) == 0) {
            x = add_nospec(x, y);
        }
    }
    return x;
}

/* Pairwise tree over the threads of a CTA (blockDim a power of two, <= 1024), thread t holding the
 * sum of the t-th aligned subtree.  Result valid in thread 0.  sh needs blockDim/32 doubles. */
__device__ __forceinline__ double cta_tree(double x, double* sh)
{
    x = warp_tree(x);
    int nw = blockDim.x >> 5;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
        sh[wid] = x;
    }
    __syncthreads();
    if (wid == 0) {
        double y = lane < nw ? sh[lane] : 0.0;
        /* pairwise over the nw warp sums (pad with zeros to 32 lanes: x + 0 is exact) */
        y = warp_tree(y);
        x = y;
    }
    return x;
}

/*
 * Two cta_tree sums at once, same trees and results as cta_tree(x) and cta_tree(y), with fewer fp64
 * instructions: the fp64 pipe takes a warp instruction whatever its active lanes, so the x and y
 * trees share instructions.  In a warp, the first level (16 x pairs and 16 y pairs) is one full-warp
 * addition leaving [x partials | y partials] in lanes 0-15 | 16-31, and each further level
 * v_l = v_2l + v_2l+1 pairs that concatenation in order (x in the lower, y in the upper half of the
 * active lanes); the CTA level does the same over [warp x sums | warp y sums].  Result valid in
 * thread 0.  sh needs 64 doubles.
 */
__device__ __forceinline__ double2 cta_tree2(double x, double y, double* sh)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    double v;
    {
        const double xa = __shfl_sync(full, x, (2 * lane) & 31), xb = __shfl_sync(full, x, (2 * lane + 1) & 31);
        const double ya = __shfl_sync(full, y, (2 * lane) & 31), yb = __shfl_sync(full, y, (2 * lane + 1) & 31);
        v = add_nospec(lane < 16 ? xa : ya, lane < 16 ? xb : yb);
    }
#pragma unroll
    for (int h = 16; h >= 2; h >>= 1) {
        const double a = __shfl_sync(full, v, (2 * lane) & 31), b = __shfl_sync(full, v, (2 * lane + 1) & 31);
        if (lane < h) {
            v = add_nospec(a, b);
        }
    }
    /* lane 0: the warp's x sum, lane 1: its y sum */
    __syncthreads();
    if (lane < 2) {
        sh[32 * lane + wid] = v;
    }
    __syncthreads();
    if (wid == 0) {
        if (nw <= 16) {
            double w = lane < nw ? sh[lane] : (lane < 2 * nw ? sh[32 + lane - nw] : 0.0);
            for (int h = nw; h >= 2; h >>= 1) {
                const double a = __shfl_sync(full, w, (2 * lane) & 31), b = __shfl_sync(full, w, (2 * lane + 1) & 31);
                if (lane < h) {
                    w = add_nospec(a, b);
                }
            }
            x = w;
            y = __shfl_sync(full, w, 1);
        }
        else {
            double a = sh[lane], b = sh[32 + lane];
#pragma unroll
            for (int m = 1; m < 32; m <<= 1) {
                const double ao = __shfl_down_sync(full, a, m), bo = __shfl_down_sync(full, b, m);
                if ((lane & (2 * m - 1)) == 0) {
                    a = add_nospec(a, ao);
                    b = add_nospec(b, bo);
                }
            }
            x = a;
            y = b;
        }
    }
    return make_double2(x, y);
}

/* Pairwise sum of v[lo .. lo+len) with len a power of two (binary-counter order == recursive tree). */
template <class F>
__device__ __forceinline__ double serial_tree(F get, int64_t lo, int64_t len)
{
    double st[40];
    for (int64_t i = 0; i < len; ++i) {
        double x = get(lo + i);
        int64_t j = i;
        int lvl = 0;
        while (j & 1) {
            x = FQ_ADD(st[lvl], x);
            j >>= 1;
            ++lvl;
        }
        st[lvl] = x;
    }
    int lvl = 0;
    while ((int64_t(1) << lvl) < len) {
        ++lvl;
    }
    return st[lvl];
}

/* serial_tree of two sums at once over len leaves (a power of two): aligned groups of 8 leaves are
 * loaded together (8 loads in flight, not one) and summed as their canonical subtree in registers,
 * then folded into the stack as above; the same additions in the same order. */
template <class F>
__device__ __forceinline__ double2 serial_tree2(F get, int64_t lo, int64_t len)
{
    if (len < 8) {
        return make_double2(serial_tree([&](int64_t i) { return get(i).x; }, lo, len),
                            serial_tree([&](int64_t i) { return get(i).y; }, lo, len));
    }
    double sx[40], sy[40];
    const int64_t nb = len / 8;
    for (int64_t b = 0; b < nb; ++b) {
        double2 q[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            q[i] = get(lo + 8 * b + i);
        }
        double x = FQ_ADD(FQ_ADD(FQ_ADD(q[0].x, q[1].x), FQ_ADD(q[2].x, q[3].x)),
                          FQ_ADD(FQ_ADD(q[4].x, q[5].x), FQ_ADD(q[6].x, q[7].x)));
        double y = FQ_ADD(FQ_ADD(FQ_ADD(q[0].y, q[1].y), FQ_ADD(q[2].y, q[3].y)),
                          FQ_ADD(FQ_ADD(q[4].y, q[5].y), FQ_ADD(q[6].y, q[7].y)));
        int64_t j = b;
        int lvl = 0;
        while (j & 1) {
            x = FQ_ADD(sx[lvl], x);
            y = FQ_ADD(sy[lvl], y);
            j >>= 1;
            ++lvl;
        }
        sx[lvl] = x;
        sy[lvl] = y;
    }
    int lvl = 0;
    while ((int64_t(1) << lvl) < nb) {
        ++lvl;
    }
    return make_double2(sx[lvl], sy[lvl]);
}

__host__ __device__ __forceinline__ int64_t next_pow2(int64_t n)
{
    int64_t p = 1;
    while (p < n) {
        p <<= 1;
    }
    return p;
}

} // namespace fqsb

#endif
