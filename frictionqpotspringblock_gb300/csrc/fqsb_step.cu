/*
 * Fused velocity-Verlet step kernels (sm_103a, FP64) and the device-side run loop.
 *
 * One launch of k_step_line / k_step_grid = one System::timeStep
 * (include/FrictionQPotSpringBlock/detail.h:1539-1570) over all particles, fused with everything
 * timeStep calls: the u update (:1549), updated_u -> potential force with the well search
 * (Cuspy::force :139-170 / SemiSmooth :236-277 / Smooth :379-409), the interaction
 * (Laplace1d::force :474-487 / Laplace2d::force :545-583), the frame force (:1353-1356), the three
 * velocity updates with damping and force sums (:1552-1565, :1321-1395) and the NaN check
 * (:1567-1569); when the run asks for it also the residual terms of minimise /
 * timeStepsUntilEvent (residual :1512-1520, StopList test :1780-1783) and the plastic-activity
 * bookkeeping (:1768-1778, :1855-1866).
 *
 * Run loop.  A run (timeSteps, flowSteps, minimise, minimise_truncate, timeStepsUntilEvent) is one
 * CUDA graph: a conditional WHILE node whose body is one step.  The last CTA to finish a step
 * evaluates the stop tests and sets the loop condition (cudaGraphSetConditional), so the host
 * launches the graph once and synchronises once.  A launch also yields after a device-time budget
 * (%globaltimer), so the host regains control every ~0.2 s of a long run.
 *
 * Chunk windows.  The step kernels only search a particle's current chunk window (a few loads).
 * When the new well lies outside the window's margins the window must move and be regenerated from
 * the particle's pcg32 stream (heavy code: distribution transforms).  That code is kept out of the
 * step kernels (it would raise them to 128 registers and cost ~12% throughput); instead the CTA is
 * marked pending, a conditional IF branch of the same graph iteration regenerates the marked
 * particles' windows (k_regen) and re-runs the marked CTAs (redo pass).  The step is a pure function
 * of the old state, so the redo reproduces exactly the reference's step.
 *
 * State is double buffered (u, v, a)[cur] -> (u, v, a)[cur ^ 1].  Arithmetic uses explicit
 * __dadd_rn / __dmul_rn in the reference's order (no fma contraction), so results equal the CPU
 * oracle bit for bit.  Only exact rewrites save fp64 issue slots (the fp64 pipe, ~1.6 instructions
 * per clock per SM on GB300, is the binding unit):
 *   - the partial sum f_frame + f_potential + f_interactions is formed once per step (it is the
 *     same in every computeForce of the step);
 *   - multiplications by parameters equal to 1 are skipped, and multiplications by powers of two
 *     (2 u, 4 u, and e.g. k_frame = 2^-22) are exponent adds on the integer pipe when the result
 *     stays normal;
 *   - the well test yl <= u < yr and the NaN test run on order-preserving integer keys.
 */
#include "fqsb_internal.h"

#include <cooperative_groups.h>

namespace fqsb {

/*
 * Resident CTAs of 256 threads per SM the step kernels are compiled for (register cap 48 at 5).  The
 * integer-pipe operations are long dependent chains; occupancy hides them (4.9 G particle-steps/s
 * slower at the 93-112 registers the compiler picks unbounded).  The Smooth potential's
 * double-double sine needs more registers than the cap allows without spilling.
 */
template <int POT>
struct StepOcc {
    static constexpr int value = POT == POT_SMOOTH ? 2 : 5;
};

template <unsigned SOFT = 0u>
__device__ __forceinline__ double u_next(const DevSys& s, const double* u0, const double* v0, const double* a0,
                                         int64_t q)
{
    return S_ADD(3, S_ADD(2, u0[q], S_MUL(0, s.dt, v0[q])), S_MUL(1, s.hdt2, a0[q]));
}

/* f = (sfi + f_damping) [+ f_thermal]: computeForce, detail.h:1321-1330 */
template <bool TH>
__device__ __forceinline__ double with_thermal(double f, double fth)
{
    return TH ? __dadd_rn(f, fth) : f;
}

/* velocity / acceleration updates of timeStep after the positions, detail.h:1552-1565 (TH: with the
 * thermal force of RandomNormalForcing as the last term of each force sum) */
template <unsigned SOFT = 0u, bool TH = false>
__device__ __forceinline__ void verlet_velocity(const DevSys& s, double sfi, double v0, double a0, double& v, double& a,
                                                double& f, double fth = 0.0)
{
    v = S_ADD(11, v0, S_MUL(10, s.dt, a0));
    f = with_thermal<TH>(S_ADD(13, sfi, S_MUL(12, s.me, v)), fth);
    a = scale(f, s.s_im);
    v = S_ADD(16, v0, S_MUL(15, s.hdt, S_ADD(14, a0, a)));
    f = with_thermal<TH>(S_ADD(18, sfi, S_MUL(17, s.me, v)), fth);
    a = scale(f, s.s_im);
    v = S_ADD(21, v0, S_MUL(20, s.hdt, S_ADD(19, a0, a)));
    f = with_thermal<TH>(S_ADD(23, sfi, S_MUL(22, s.me, v)), fth);
    a = scale(f, s.s_im);
}

/* (f_frame + f_potential) of the force sum, and f_frame itself */
template <int POT, unsigned SOFT = 0u>
__device__ __forceinline__ double frame_pot(const DevSys& s, const double4_32a& w, double up, double uf, double& ff)
{
    double fp = pot_force<POT, SOFT>(s, w, up);
    ff = scale(S_SUB(4, uf, up), s.s_kf);
    return S_ADD(6, ff, fp);
}

__device__ __forceinline__ long long absll(long long x)
{
    return x < 0 ? -x : x;
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void set_loop(const DevSys& s, unsigned v)
{
    if (s.in_graph) {
        cudaGraphSetConditional((cudaGraphConditionalHandle)s.h_while, v);
    }
}

__device__ __forceinline__ void set_branch(const DevSys& s, unsigned v)
{
    if (s.in_graph) {
        cudaGraphSetConditional((cudaGraphConditionalHandle)s.h_if, v);
    }
}

/*
 * Bookkeeping and stop tests of one finished step on a run-control block c (global memory for the
 * graph path, shared memory for the one-cluster path) and its StopList window `ring`: step and
 * increment counters, frame position, plastic activity, NaN / yield-search errors, the StopList
 * residual test (GooseFEM::Iterate::StopList, detail.h:1780-1783), event, truncation and step limits.
 */
template <typename CTL>
__device__ __forceinline__ void finalize_ctl(CTL* c, double* ring, double uf, double sf, double sff)
{
    int flags = c->flags;
    c->ticket = 0;
    c->ticket_redo = 0;
    c->n_pending_cta = 0;
    c->n_regen = 0;
    if (flags & RF_FFSUM) {
        c->rec_ffsum[c->step] = sf;
    }
    if (flags & RF_SCHEDULE) {
        c->u_frame = uf;
    }
    c->step += 1;
    if (!(flags & RF_NOINC)) {
        c->inc += 1;
    }
    c->cur ^= 1;
    if (flags & RF_FLOW) {
        c->u_frame = uf;
    }
    uint64_t now = globaltimer();
    if (c->launch_steps == 0) {
        c->launch_t0 = now;
    }
    c->launch_steps += 1;
    if (c->nan_flag) {
        c->error = DERR_NAN;
    }
    else if (c->walk_flag) {
        c->error = DERR_WALK;
    }
    else {
        if (flags & (RF_ACT | RF_TRUNCATE)) {
            long long sv = c->s_sum;
            if (sv != c->s_n) {
                if (c->init) {
                    c->init = 0;
                    c->qs_first = c->inc;
                }
                c->qs_last = c->inc;
            }
            c->s_n = sv;
        }
        if ((flags & RF_EVENT) && c->a_count != 0) {
            c->done = RUN_EVENT;
        }
        if (!c->done && (flags & RF_RESID)) {
            double r_fres = FQ_SQRT(sf);
            double r_fext = FQ_SQRT(sff);
            double r = r_fext != 0.0 ? FQ_DIV(r_fres, r_fext) : r_fres;
            c->last_residual = r;
            int64_t n = c->niter_tol;
            if (n > 0) {
                int64_t pos = c->sl_pos;
                double old = ring[pos];
                if (old >= c->tol) {
                    c->sl_ge_tol -= 1;
                }
                if (old >= c->tol2) {
                    c->sl_ge_tol2 -= 1;
                }
                if (n >= 2) {
                    double second = ring[(pos + 1) % n];
                    if (second > old) {
                        c->sl_asc -= 1;
                    }
                    double newest = ring[(pos + n - 1) % n];
                    if (r > newest) {
                        c->sl_asc += 1;
                    }
                }
                ring[pos] = r;
                c->sl_pos = (pos + 1) % n;
                if (r >= c->tol) {
                    c->sl_ge_tol += 1;
                }
                if (r >= c->tol2) {
                    c->sl_ge_tol2 += 1;
                }
            }
            if ((c->sl_asc == 0 && c->sl_ge_tol == 0) || c->sl_ge_tol2 == 0) {
                c->done = RUN_CONVERGED;
            }
        }
        if (!c->done && (flags & RF_TRUNCATE)) {
            if ((c->A_truncate > 0 && c->a_count >= c->A_truncate) ||
                (c->S_truncate > 0 && c->s_sum >= c->S_truncate)) {
                c->done = RUN_TRUNCATED;
            }
        }
        if (!c->done && c->step >= c->max_steps) {
            c->done = RUN_MAXITER;
        }
    }
}

/*
 * Stop tests of one finished step (thread 0 of the CTA that finishes the step last); sets the
 * run-loop condition.  sf / sff: sum of f^2 and of f_frame^2 over all particles.
 */
__device__ void finalize_step(const DevSys& s, double uf, double sf, double sff)
{
    Ctl* c = s.ctl;
    finalize_ctl(c, s.ring, uf, sf, sff);
    bool more = !c->done && !c->error && (globaltimer() - c->launch_t0) < c->budget_ns;
    __threadfence();
    set_loop(s, more ? 1u : 0u);
}

/* Whole-CTA canonical tree over partials[0..G) (zero padded to a power of two). */
static __device__ __noinline__ double2 tree_partials(const double2* partials, int64_t G, double* sh)
{
    int64_t P = next_pow2(G);
    int T = blockDim.x;
    double x = 0.0, y = 0.0;
    if (P <= T) {
        if (threadIdx.x < G) {
            double2 q = __ldcg(partials + threadIdx.x);
            x = q.x;
            y = q.y;
        }
    }
    else {
        int64_t per = P / T;
        int64_t lo = (int64_t)threadIdx.x * per;
        const double2 t = serial_tree2(
            [&](int64_t i) { return i < G ? __ldcg(partials + i) : make_double2(0.0, 0.0); }, lo, per);
        x = t.x;
        y = t.y;
    }
    return cta_tree2(x, y, sh);
}

struct StepShared {
    int exit_flag;
    int cur;
    int flags;
    int last;
    int nan;
    int pending;
    double uf;
    unsigned long long ds;
    unsigned long long da;
    double red[64];
};

/* Reads the run state; returns false when the run is already over (then CTA 0 ends the loop). */
__device__ __forceinline__ bool step_prologue(const DevSys& s, StepShared& sh, bool graph_loop)
{
    int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if (tid == 0) {
        volatile Ctl* c = s.ctl;
        sh.exit_flag = (c->done != 0) || (c->error != 0);
        sh.cur = c->cur;
        sh.flags = c->flags;
        double uf = c->u_frame;
        if (sh.flags & RF_FLOW) {
            uf = FQ_ADD(uf, c->vdt);
        }
        if (sh.flags & RF_SCHEDULE) {
            uf = c->sched[c->step];
        }
        sh.uf = uf;
        sh.nan = 0;
        sh.pending = 0;
        sh.ds = 0ull;
        sh.da = 0ull;
        sh.last = 0;
        if (sh.exit_flag && graph_loop && blockIdx.x == 0 && blockIdx.y == 0) {
            set_loop(s, 0u);
        }
    }
    __syncthreads();
    return sh.exit_flag == 0;
}

/*
 * Searches particle p's current chunk window for the well of u (y[i] <= u < y[i+1], the prrng
 * align rule) and commits it when it lies inside the window's margins [min_margin, W - buffer).
 * Returns false when the window must move (then nothing is changed).
 */
__device__ __forceinline__ bool window_search(const DevSys& s, int64_t p, double u, double4_32a& w)
{
    const int64_t W = s.W;
    const double* y = s.data + p * W;
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
    if (li < s.min_margin || li >= W - s.buffer) {
        return false;
    }
    s.cidx[p] = (int32_t)li;
    s.gidx[p] = s.start[p] + li;
    w = make_wc(s, y[li], y[li + 1]);
    s.wc[p] = w;
    return true;
}

__device__ __forceinline__ bool non_finite(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) >= 0x7ff0000000000000LL;
}

/*
 * Per-particle well check of the cached well w (particle p's record, loaded by the caller); returns the
 * (possibly refreshed) well cache.  `regen` is set when the particle's chunk window must move; the
 * pass-1 caller then marks its CTA pending.
 */
__device__ __forceinline__ double4_32a well_of(const DevSys& s, int64_t p, double un, bool act, StepShared& sh,
                                               bool& regen, double4_32a w)
{
    regen = false;
    if (!in_well(w.x, w.y, un) && !non_finite(un)) {
        int64_t gold = s.gidx[p];
        if (window_search(s, p, un, w)) {
            int64_t gnew = s.gidx[p];
            if (act && gnew != gold) {
                int64_t ref = s.i_n[p];
                long long ds = absll(gnew - ref) - absll(gold - ref);
                long long da = (long long)(gnew != ref) - (long long)(gold != ref);
                atomicAdd(&sh.ds, (unsigned long long)ds);
                atomicAdd(&sh.da, (unsigned long long)da);
            }
        }
        else {
            regen = true;
        }
    }
    return w;
}

__device__ __forceinline__ double4_32a well_of(const DevSys& s, int64_t p, double un, bool act, StepShared& sh,
                                               bool& regen)
{
    return well_of(s, p, un, act, sh, regen, s.wc[p]);
}

/* Role of the CTA epilogue in the step's kernels. */
enum : int {
    EPI_LINE = 0,      /* 1d pass 1: last CTA finalises, or opens the regeneration branch */
    EPI_GRID_STEP = 1, /* 2d pass 1: last CTA opens (or closes) the regeneration branch */
    EPI_REDO = 2,      /* 1d redo of the pending CTAs: the last of them finalises */
    EPI_REDUCE = 3     /* 2d reduction: last CTA finalises */
};

/*
 * End of a CTA's part of a step: commits activity / NaN flags and the CTA's residual subtree; the CTA
 * that finishes last (ticket) finalises the step or steers the regeneration branch, per `mode`.
 */
__device__ __forceinline__ void step_epilogue(const DevSys& s, StepShared& sh, int mode, double rf, double rff)
{
    const bool resid = (sh.flags & (RF_RESID | RF_FFSUM)) != 0;
    const bool tree = resid && mode != EPI_GRID_STEP;
    double sf = 0.0, sff = 0.0;
    if (tree) {
        double2 t = cta_tree2(rf, rff, sh.red);
        sf = t.x;
        sff = t.y;
    }
    __syncthreads();
    int tid = threadIdx.x + threadIdx.y * blockDim.x;
    int64_t bid = blockIdx.x + (int64_t)blockIdx.y * gridDim.x;
    Ctl* c = s.ctl;
    if (tid == 0) {
        if (tree) {
            s.partials[bid] = make_double2(sf, sff);
        }
        if (sh.ds) {
            atomicAdd((unsigned long long*)&c->s_sum, sh.ds);
        }
        if (sh.da) {
            atomicAdd((unsigned long long*)&c->a_count, sh.da);
        }
        if (sh.nan && !sh.pending) {
            atomicOr(&c->nan_flag, 1);
        }
        if (sh.pending) {
            s.cta_pending[bid] = 1;
            atomicAdd(&c->n_pending_cta, 1);
        }
        __threadfence();
        if (mode == EPI_REDO) {
            unsigned t = atomicAdd(&c->ticket_redo, 1u);
            sh.last = (t == (unsigned)c->n_pending_cta - 1u) ? 1 : 0;
        }
        else {
            unsigned t = atomicAdd(&c->ticket, 1u);
            sh.last = (t == gridDim.x * gridDim.y - 1) ? 1 : 0;
        }
    }
    __syncthreads();
    if (!sh.last) {
        return;
    }
    __threadfence();
    if (mode == EPI_LINE || mode == EPI_GRID_STEP) {
        bool pend = c->n_pending_cta > 0;
        if (pend || mode == EPI_GRID_STEP) {
            if (tid == 0) {
                c->ticket = 0;
                set_branch(s, pend ? 1u : 0u);
            }
            return;
        }
        if (tid == 0) {
            set_branch(s, 0u);
        }
    }
    double2 tot = make_double2(0.0, 0.0);
    if (resid) {
        tot = tree_partials(s.partials, (int64_t)gridDim.x * gridDim.y, sh.red);
    }
    if (tid == 0) {
        finalize_step(s, sh.uf, tot.x, tot.y);
    }
}

/*
 * Line1d (INTER_LAPLACE1D) or Particles (INTER_NONE) step.  Thread t of CTA b owns the PPT consecutive
 * particles b*T*PPT + t*PPT + [0, PPT): a CTA covers an aligned power-of-two range of the flat index,
 * so the residual sums follow the fixed pairwise tree over the flat index.  Updated positions are
 * exchanged through shared memory (one barrier); the two particles just outside the CTA are recomputed
 * from the old state.  State arrays are padded to a multiple of 1024 entries.  redo = 1: only CTAs
 * marked pending run (after k_regen moved their particles' windows).
 */
template <int POT, int INTER, int PPT, unsigned SOFT = STEP_SOFT, bool TH = false, int MODE = KMODE_GENERAL>
__global__ void __launch_bounds__(256, StepOcc<POT>::value) k_step_line(DevSys s, int redo)
{
    __shared__ StepShared sh;
    __shared__ double sh_un[256 * PPT];
    __shared__ double sh_halo[2]; /* ring neighbours left of the tile's first particle, right of its last */
    if (!step_prologue(s, sh, true)) {
        return;
    }
    if (redo) {
        if (!s.cta_pending[blockIdx.x]) {
            return;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s.cta_pending[blockIdx.x] = 0;
        }
    }
    const int cur = sh.cur;
    /* KMODE_PLAIN: the instantiation for runs without activity, residual, frame-force sums or recording
     * (timeSteps / flowSteps); KMODE_RESID: with the residual only (minimise); the rest compiled out */
    const bool general = MODE == KMODE_GENERAL;
    const bool act = general && (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = MODE == KMODE_RESID || (general && (sh.flags & RF_RESID) != 0);
    const bool ffsum = general && (sh.flags & RF_FFSUM) != 0;
    const bool record = general && (sh.flags & RF_RECORD) != 0;
    const int64_t rec_step = record ? ((volatile Ctl*)s.ctl)->step : 0;
    const double uf = sh.uf;
    const int64_t N = s.N;
    const int T = blockDim.x;
    const int64_t base = (int64_t)blockIdx.x * T * PPT;
    const int64_t p0 = base + (int64_t)threadIdx.x * PPT;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    double* u1 = s.u[cur ^ 1];
    double* v1 = s.v[cur ^ 1];
    double* a1 = s.a[cur ^ 1];

    double un[PPT], vr[PPT], ar[PPT];
    /* the cached wells are loaded together with the state, so that their latency overlaps the
     * position update and the neighbour exchange instead of following them */
    double4_32a wpre[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        if (p0 + j < N) {
            wpre[j] = s.wc[p0 + j];
        }
    }
    if (PPT == 2) {
        double2 uu = *reinterpret_cast<const double2*>(u0 + p0);
        double2 vv = *reinterpret_cast<const double2*>(v0 + p0);
        double2 aa = *reinterpret_cast<const double2*>(a0 + p0);
        vr[0] = vv.x;
        vr[PPT - 1] = vv.y;
        ar[0] = aa.x;
        ar[PPT - 1] = aa.y;
        un[0] = S_ADD(3, S_ADD(2, uu.x, S_MUL(0, s.dt, vr[0])), S_MUL(1, s.hdt2, ar[0]));
        un[PPT - 1] = S_ADD(3, S_ADD(2, uu.y, S_MUL(0, s.dt, vr[PPT - 1])), S_MUL(1, s.hdt2, ar[PPT - 1]));
    }
    else {
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            vr[j] = v0[p0 + j];
            ar[j] = a0[p0 + j];
            un[j] = S_ADD(3, S_ADD(2, u0[p0 + j], S_MUL(0, s.dt, vr[j])), S_MUL(1, s.hdt2, ar[j]));
        }
    }
    if (inter_ring(INTER)) {
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            sh_un[threadIdx.x * PPT + j] = un[j];
        }
        if (threadIdx.x < 2) {
            /* the two neighbours outside the tile, recomputed from the old state by two lanes of one
             * warp (one pass through the position update instead of one in each of two warps) */
            const int64_t last = (base + (int64_t)T * PPT < N ? base + (int64_t)T * PPT : N) - 1;
            const int64_t q = threadIdx.x == 0 ? (base == 0 ? N - 1 : base - 1) : (last + 1 == N ? 0 : last + 1);
            sh_halo[threadIdx.x] = u_next(s, u0, v0, a0, q);
        }
        __syncthreads();
    }
    double rf = 0.0, rff = 0.0;
    bool nan = false, pending = false;
    double vo[PPT], ao[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        int64_t p = p0 + j;
        vo[j] = 0.0;
        ao[j] = 0.0;
        if (p >= N) {
            continue;
        }
        double up = un[j];
        bool regen;
        double4_32a w = well_of(s, p, up, act, sh, regen, wpre[j]);
        pending |= regen;
        double ff;
        double sfp = frame_pot<POT, SOFT>(s, w, up, uf, ff);
        double fi = 0.0;
        if (inter_ring(INTER)) {
            int li = threadIdx.x * PPT + j;
            double uL = li > 0 ? sh_un[li - 1] : sh_halo[0];
            double uR = (li + 1 < T * PPT && p + 1 < N) ? sh_un[li + 1] : sh_halo[1];
            fi = ring_force<INTER, SOFT>(s, uL, up, uR);
        }
        double sfi = S_ADD(9, sfp, fi);
        double f;
        verlet_velocity<SOFT, TH>(s, sfi, vr[j], ar[j], vo[j], ao[j], f, TH ? s.f_th[p] : 0.0);
        nan |= is_nan_bits(up);
        if (resid) {
            /* squares on the integer pipes (bit-identical), sums on the fp64 pipe */
            double f2 = fq_smul(f, f), ff2 = fq_smul(ff, ff);
            if (j == 0) {
                rf = f2;
                rff = ff2;
            }
            else {
                rf = add_nospec(rf, f2);
                rff = add_nospec(rff, ff2);
            }
        }
        else if (ffsum) {
            rf = j == 0 ? ff : add_nospec(rf, ff);
        }
        if (record) {
            size_t o = (size_t)rec_step * (size_t)N + (size_t)p;
            s.ctl->rec_u[o] = up;
            s.ctl->rec_v[o] = vo[j];
            s.ctl->rec_a[o] = ao[j];
            s.ctl->rec_w[o] = w;
        }
    }
    if (p0 < N) {
        if (PPT == 2) {
            *reinterpret_cast<double2*>(u1 + p0) = make_double2(un[0], un[PPT - 1]);
            *reinterpret_cast<double2*>(v1 + p0) = make_double2(vo[0], vo[PPT - 1]);
            *reinterpret_cast<double2*>(a1 + p0) = make_double2(ao[0], ao[PPT - 1]);
        }
        else {
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                u1[p0 + j] = un[j];
                v1[p0 + j] = vo[j];
                a1[p0 + j] = ao[j];
            }
        }
    }
    if (nan) {
        sh.nan = 1;
    }
    if (pending && !redo) {
        sh.pending = 1;
        for (int j = 0; j < PPT; ++j) {
            /* record the particles of this thread that need a new window */
            int64_t p = p0 + j;
            if (p < N) {
                double4_32a w = s.wc[p];
                if (!in_well(w.x, w.y, un[j]) && !non_finite(un[j])) {
                    int k = atomicAdd(&s.ctl->n_regen, 1);
                    s.regen_list[k] = (int32_t)p;
                }
            }
        }
    }
    if (pending && redo) {
        /* the window could not be moved (yield search bound): reported by the finalisation */
        atomicOr(&s.ctl->walk_flag, 1);
    }
    step_epilogue(s, sh, redo ? EPI_REDO : EPI_LINE, rf, rff);
}

/*
 * Line2d step: CTA tile of 8 rows x 32 columns, one particle per thread, the neighbourhood read from
 * a haloed shared tile (the halo of 84 positions recomputed by three whole warps).  The residual terms are
 * written per particle (sq2) and summed in the flat-index pairwise order by k_reduce_grid, which
 * also finalises the step.
 */
template <int POT, int INTER = INTER_LAPLACE2D, unsigned SOFT = STEP_SOFT>
__global__ void __launch_bounds__(256, StepOcc<POT>::value) k_step_grid(DevSys s, int redo)
{
    __shared__ StepShared sh;
    /* the tile's new positions at [1 + row][1 + column], with the halo around its nr x nc valid
     * particles: rows 0 and 1 + nr, columns 0 and 1 + nc, and the four corners */
    __shared__ double sh_un[10][34];
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const int64_t bid = blockIdx.x + (int64_t)blockIdx.y * gridDim.x;
    if (redo) {
        if (!s.cta_pending[bid]) {
            return;
        }
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            s.cta_pending[bid] = 0;
        }
    }
    const int cur = sh.cur;
    const bool act = (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (sh.flags & RF_RESID) != 0;
    const double uf = sh.uf;
    const int64_t R = s.rows, C = s.cols;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t row0 = (int64_t)blockIdx.y * 8, col0 = (int64_t)blockIdx.x * 32;
    const int nr = (int)(R - row0 < 8 ? R - row0 : 8);
    const int nc = (int)(C - col0 < 32 ? C - col0 : 32);
    const int64_t i = row0 + ty;
    const int64_t jc = col0 + tx;
    const bool valid = i < R && jc < C;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    const int64_t p = i * C + jc;
    double up = 0.0, vr = 0.0, ar = 0.0;
    if (valid) {
        vr = v0[p];
        ar = a0[p];
        up = S_ADD(3, S_ADD(2, u0[p], S_MUL(0, s.dt, vr)), S_MUL(1, s.hdt2, ar));
        sh_un[1 + ty][1 + tx] = up;
    }
    {
        /* the halo, recomputed from the old state (periodic) by whole warps: warp 0 the row above,
         * warp 1 the row below, warp 2 the side columns (lanes 0-7 left, 8-15 right) and the corners
         * (lanes 16-19) */
        const int64_t rt = (row0 + R - 1) % R, rb = (row0 + nr) % R;
        const int64_t cl = (col0 + C - 1) % C, cr = (col0 + nc) % C;
        if (ty == 0 && tx < nc) {
            sh_un[0][1 + tx] = u_next(s, u0, v0, a0, rt * C + jc);
        }
        else if (ty == 1 && tx < nc) {
            sh_un[1 + nr][1 + tx] = u_next(s, u0, v0, a0, rb * C + jc);
        }
        else if (ty == 2 && tx < 20) {
            int r, c;
            int64_t q;
            if (tx < 16) {
                const int k = tx & 7;
                r = 1 + k;
                c = tx < 8 ? 0 : 1 + nc;
                q = (row0 + k) * C + (tx < 8 ? cl : cr);
            }
            else {
                const int k = tx - 16;
                r = k < 2 ? 0 : 1 + nr;
                c = (k & 1) ? 1 + nc : 0;
                q = (k < 2 ? rt : rb) * C + ((k & 1) ? cr : cl);
            }
            if (tx >= 16 || (tx & 7) < nr) {
                sh_un[r][c] = u_next(s, u0, v0, a0, q);
            }
        }
    }
    __syncthreads();
    if (valid) {
        bool regen;
        double4_32a w = well_of(s, p, up, act, sh, regen);
        if (regen) {
            if (!redo) {
                sh.pending = 1;
                int k = atomicAdd(&s.ctl->n_regen, 1);
                s.regen_list[k] = (int32_t)p;
            }
            else {
                atomicOr(&s.ctl->walk_flag, 1);
            }
        }
        double ff;
        double sfp = frame_pot<POT, SOFT>(s, w, up, uf, ff);
        double fi;
        if (INTER == INTER_LAPLACE2D) {
            const double uU = sh_un[ty][1 + tx];
            const double uD = sh_un[ty + 2][1 + tx];
            const double uL = sh_un[1 + ty][tx];
            const double uR = sh_un[1 + ty][tx + 2];
            fi = scale(FQ_SUB(FQ_ADD(FQ_ADD(FQ_ADD(uU, uD), uL), uR), scale_pow2(up, 2, 4.0)), s.s_k);
        }
        else {
            /* 3 x 3 neighbourhood from the haloed tile */
            auto nb = [&](int di, int dj) -> double { return sh_un[1 + ty + di][1 + tx + dj]; };
            fi = qg2d_force(s, up, nb(1, 0), nb(-1, 0), nb(0, 1), nb(0, -1), nb(1, 1), nb(1, -1), nb(-1, 1), nb(-1, -1));
        }
        double sfi = S_ADD(9, sfp, fi);
        double vv, aa, f;
        verlet_velocity<SOFT>(s, sfi, vr, ar, vv, aa, f);
        s.u[cur ^ 1][p] = up;
        s.v[cur ^ 1][p] = vv;
        s.a[cur ^ 1][p] = aa;
        if (is_nan_bits(up)) {
            sh.nan = 1;
        }
        if (resid) {
            s.sq2[p] = make_double2(fq_smul(f, f), fq_smul(ff, ff));
        }
    }
    if (redo) {
        /* the reduction kernel after the branch finalises; only the counters are committed here */
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (sh.ds) {
                atomicAdd((unsigned long long*)&s.ctl->s_sum, sh.ds);
            }
            if (sh.da) {
                atomicAdd((unsigned long long*)&s.ctl->a_count, sh.da);
            }
            if (sh.nan) {
                atomicOr(&s.ctl->nan_flag, 1);
            }
        }
        return;
    }
    step_epilogue(s, sh, EPI_GRID_STEP, 0.0, 0.0);
}

/*
 * Line2d Laplace2d step with two rows per thread: CTA tile of 16 rows x 32 columns (blockDim 32 x 8,
 * thread (x, y) owns rows 2y and 2y + 1 of column x).  All four neighbours come from shared memory:
 * the tile's new positions and a recomputed halo of 96 positions per 512 particles, computed by three
 * whole warps (the 8 x 32 tiles of k_step_grid recompute their side columns in one lane per warp and
 * row).  Per particle the same operations in the same order as k_step_grid, so the same results.
 */
template <int POT, unsigned SOFT = STEP_SOFT>
__global__ void __launch_bounds__(256, StepOcc<POT>::value) k_step_grid2(DevSys s, int redo)
{
    __shared__ StepShared sh;
    /* the tile's new positions at [1 + row][1 + column], with the four halo lines around them: row 0
     * and row 1 + nr (the rows above and below the tile's nr valid rows), column 0 and column 1 + nc */
    __shared__ double sh_un[18][34];
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const int64_t bid = blockIdx.x + (int64_t)blockIdx.y * gridDim.x;
    if (redo) {
        if (!s.cta_pending[bid]) {
            return;
        }
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            s.cta_pending[bid] = 0;
        }
    }
    const int cur = sh.cur;
    const bool act = (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (sh.flags & RF_RESID) != 0;
    const double uf = sh.uf;
    const int64_t R = s.rows, C = s.cols;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t row0 = (int64_t)blockIdx.y * 16, col0 = (int64_t)blockIdx.x * 32;
    const int nr = (int)(R - row0 < 16 ? R - row0 : 16);
    const int nc = (int)(C - col0 < 32 ? C - col0 : 32);
    const int64_t jc = col0 + tx;
    const int64_t i0 = row0 + 2 * ty;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    double up[2], vr[2], ar[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int64_t i = i0 + q;
        up[q] = vr[q] = ar[q] = 0.0;
        if (i < R && jc < C) {
            const int64_t p = i * C + jc;
            vr[q] = v0[p];
            ar[q] = a0[p];
            up[q] = S_ADD(3, S_ADD(2, u0[p], S_MUL(0, s.dt, vr[q])), S_MUL(1, s.hdt2, ar[q]));
            sh_un[1 + 2 * ty + q][1 + tx] = up[q];
        }
    }
    /* the halo, recomputed from the old state (periodic): warp 0 the row above, warp 1 the row below,
     * warp 2 the columns left (lanes 0-15) and right (lanes 16-31); whole warps, no divergent lanes */
    if (ty == 0 && tx < nc) {
        sh_un[0][1 + tx] = u_next(s, u0, v0, a0, ((row0 + R - 1) % R) * C + jc);
    }
    else if (ty == 1 && tx < nc) {
        sh_un[1 + nr][1 + tx] = u_next(s, u0, v0, a0, ((row0 + nr) % R) * C + jc);
    }
    else if (ty == 2 && (tx & 15) < nr) {
        const int r = tx & 15;
        const int64_t c = tx < 16 ? (col0 + C - 1) % C : (col0 + nc) % C;
        sh_un[1 + r][tx < 16 ? 0 : 1 + nc] = u_next(s, u0, v0, a0, (row0 + r) * C + c);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int64_t i = i0 + q;
        if (!(i < R && jc < C)) {
            continue;
        }
        const int64_t p = i * C + jc;
        const int r = 2 * ty + q;
        bool regen;
        double4_32a w = well_of(s, p, up[q], act, sh, regen);
        if (regen) {
            if (!redo) {
                sh.pending = 1;
                int k = atomicAdd(&s.ctl->n_regen, 1);
                s.regen_list[k] = (int32_t)p;
            }
            else {
                atomicOr(&s.ctl->walk_flag, 1);
            }
        }
        double ff;
        double sfp = frame_pot<POT, SOFT>(s, w, up[q], uf, ff);
        const double uU = sh_un[r][1 + tx];
        const double uD = sh_un[r + 2][1 + tx];
        const double uL = sh_un[1 + r][tx];
        const double uR = sh_un[1 + r][tx + 2];
        double fi = scale(FQ_SUB(FQ_ADD(FQ_ADD(FQ_ADD(uU, uD), uL), uR), scale_pow2(up[q], 2, 4.0)), s.s_k);
        double sfi = S_ADD(9, sfp, fi);
        double vv, aa, f;
        verlet_velocity<SOFT>(s, sfi, vr[q], ar[q], vv, aa, f);
        s.u[cur ^ 1][p] = up[q];
        s.v[cur ^ 1][p] = vv;
        s.a[cur ^ 1][p] = aa;
        if (is_nan_bits(up[q])) {
            sh.nan = 1;
        }
        if (resid) {
            s.sq2[p] = make_double2(fq_smul(f, f), fq_smul(ff, ff));
        }
    }
    if (redo) {
        /* the reduction kernel after the branch finalises; only the counters are committed here */
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            if (sh.ds) {
                atomicAdd((unsigned long long*)&s.ctl->s_sum, sh.ds);
            }
            if (sh.da) {
                atomicAdd((unsigned long long*)&s.ctl->a_count, sh.da);
            }
            if (sh.nan) {
                atomicOr(&s.ctl->nan_flag, 1);
            }
        }
        return;
    }
    step_epilogue(s, sh, EPI_GRID_STEP, 0.0, 0.0);
}

/* Rows of a CTA tile of the 2d step kernel: 16 for Laplace2d (k_step_grid2), 8 otherwise. */
static int64_t grid_tile_rows(const DevSys& s)
{
    return s.inter == INTER_LAPLACE2D ? 16 : 8;
}

/* Pairwise reduction of the 2d step's sq2 in flat-index order (1024 per CTA) + step finalisation. */
__global__ void __launch_bounds__(256) k_reduce_grid(DevSys s)
{
    __shared__ StepShared sh;
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const bool resid = (sh.flags & RF_RESID) != 0;
    double rf = 0.0, rff = 0.0;
    if (resid) {
        int64_t lo = (int64_t)blockIdx.x * 1024 + threadIdx.x * 4;
        double x[4], y[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (lo + j < s.N) {
                double2 q = s.sq2[lo + j];
                x[j] = q.x;
                y[j] = q.y;
            }
            else {
                x[j] = 0.0;
                y[j] = 0.0;
            }
        }
        rf = FQ_ADD(FQ_ADD(x[0], x[1]), FQ_ADD(x[2], x[3]));
        rff = FQ_ADD(FQ_ADD(y[0], y[1]), FQ_ADD(y[2], y[3]));
    }
    step_epilogue(s, sh, EPI_REDUCE, rf, rff);
}

/* Regeneration branch: move the chunk windows of the particles recorded by pass 1. */
__global__ void __launch_bounds__(128) k_regen(DevSys s)
{
    Ctl* c = s.ctl;
    if (c->done || c->error) {
        return;
    }
    const int cur = c->cur;
    const bool act = (c->flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const int n = c->n_regen;
    auto count_move = [&](int64_t p, int64_t gold) {
        int64_t gnew = s.gidx[p];
        if (act && gnew != gold) {
            int64_t ref = s.i_n[p];
            long long ds = absll(gnew - ref) - absll(gold - ref);
            long long da = (long long)(gnew != ref) - (long long)(gold != ref);
            atomicAdd((unsigned long long*)&c->s_sum, (unsigned long long)ds);
            atomicAdd((unsigned long long*)&c->a_count, (unsigned long long)da);
        }
    };
    if (n >= (int)(gridDim.x * blockDim.x) / 4) {
        /* many moves: one thread per particle keeps every thread busy */
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            int64_t p = s.regen_list[k];
            int64_t gold = s.gidx[p];
            dev_align(s, p, u_next(s, s.u[cur], s.v[cur], s.a[cur], p));
            count_move(p, gold);
        }
        return;
    }
    /* few moves: one CTA per particle, its threads sharing the draws (fwd_move_*); the same values */
    __shared__ FwdMove m_sh;
    __shared__ int ok_sh;
    __shared__ long long gold_sh;
    const uint64_t mv_c = pcg_advance(0ULL, (uint64_t)blockDim.x);
    const uint64_t mv_a = pcg_advance(1ULL, (uint64_t)blockDim.x) - mv_c;
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        const int64_t p = s.regen_list[k];
        if (threadIdx.x == 0) {
            double un = u_next(s, s.u[cur], s.v[cur], s.a[cur], p);
            gold_sh = s.gidx[p];
            FwdMove m;
            ok_sh = fwd_move_plan(s, p, un, m) ? 1 : 0;
            if (ok_sh) {
                m_sh = m;
            }
            else {
                dev_align(s, p, un);
            }
        }
        __syncthreads();
        if (ok_sh) {
            fwd_move_draws(s, m_sh, (int)threadIdx.x, (int)blockDim.x, mv_a, mv_c);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (ok_sh) {
                fwd_move_sum(s, m_sh);
            }
            count_move(p, gold_sh);
        }
        __syncthreads();
    }
}

/*
 * Next-window buffers of a small system, refreshed before a run of the one-cluster kernel: each CTA
 * takes particles blockIdx.x, blockIdx.x + gridDim.x, ...; a particle whose buffer does not follow
 * its current window (next_window_ready) gets the W draws after the window end from all the CTA's
 * threads, then their running sum from one thread.  A particle whose buffer is current costs one
 * comparison, so the kernel is cheap when few windows moved.
 */
__global__ void __launch_bounds__(128) k_next_window(DevSys s)
{
    __shared__ int need_sh, kind_sh;
    __shared__ uint64_t st_sh;
    __shared__ long long end_sh;
    const uint64_t mv_c = pcg_advance(0ULL, (uint64_t)blockDim.x);
    const uint64_t mv_a = pcg_advance(1ULL, (uint64_t)blockDim.x) - mv_c;
    for (int64_t p = blockIdx.x; p < s.N; p += gridDim.x) {
        if (threadIdx.x == 0) {
            const int64_t end = s.start[p] + s.W - 1;
            int kind;
            int64_t ko;
            uint64_t sto;
            need_sh = s.nx_end[p] != end && next_window_applies(s, p, end, kind, ko, sto);
            if (need_sh) {
                kind_sh = kind;
                end_sh = end;
                st_sh = pcg_advance(sto, (uint64_t)(end + 1 - ko));
            }
        }
        __syncthreads();
        if (need_sh) {
            seq_draws(s, s.nx + p * s.W, s.W, st_sh, (int)threadIdx.x, (int)blockDim.x, mv_a, mv_c);
            __syncthreads();
            if (threadIdx.x == 0) {
                next_window_sum(s, p, end_sh, kind_sh);
                s.nx_end[p] = end_sh;
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_next_window(const DevSys& s, cudaStream_t st)
{
    if (s.nx == nullptr) {
        return cudaSuccess;
    }
    const int64_t grid = s.N < 4 * 152 ? s.N : 4 * 152;
    k_next_window<<<(unsigned)grid, 128, 0, st>>>(s);
    return cudaGetLastError();
}

/* ------------------------------------------------------------- thermal forcing */

/*
 * RandomNormalForcing::force (detail.h:930-942), run by updated_inc at the start of every time step
 * (timeStep :1540-1544) and by refresh / set_inc: in particle order, every particle with inc >= next[p]
 * takes the next draw of one pcg32 stream, f_thermal[p] = mean + (stddev sqrt 2) erfinv(2 r - 1)
 * (r = u32 2^-32), and next[p] += dinc[p].  The draws are numbered by an exclusive scan over the flat
 * index: k_th_count counts each 1024-particle tile's draws and its last CTA turns the counts into
 * tile offsets and jumps the stream past the whole draw; k_th_list writes each drawing particle to
 * its rank in a compact list; k_th_eval gives list entry k the k-th output after the old state (a
 * jump-ahead per entry) with one thread per draw, so the erfinv work is dense whatever the fraction
 * of particles that draw, and the result equals the reference's sequential loop.
 *
 * from_ctl = 1: inside a run, for the step about to run (inc = Ctl::inc + 1); nothing happens once the
 * run is over or when the run's iterations are not time steps.  from_ctl = 0: at inc = inc_arg.
 */
constexpr int TH_TILE = 1024; /* particles per CTA of the draw kernels: 256 threads x 4 */

__device__ __forceinline__ bool th_draw_inc(const DevSys& s, int from_ctl, int64_t inc_arg, int64_t& inc)
{
    if (!from_ctl) {
        inc = inc_arg;
        return true;
    }
    volatile Ctl* c = s.ctl;
    if (c->done || c->error || (c->flags & RF_NOINC)) {
        return false;
    }
    inc = c->inc + 1;
    return true;
}

/* Exclusive prefix of x over the CTA's 256 threads (8 warps); *total gets the CTA's sum. */
__device__ __forceinline__ int64_t cta_exclusive_scan256(int64_t x, int64_t* sh8, int64_t* total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) {
            incl += y;
        }
    }
    if (lane == 31) {
        sh8[warp] = incl;
    }
    __syncthreads();
    int64_t before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        int64_t t = sh8[w];
        before += w < warp ? t : 0;
        all += t;
    }
    __syncthreads();
    *total = all;
    return before + incl - x;
}

__global__ void __launch_bounds__(256) k_th_count(DevSys s, int from_ctl, int64_t inc_arg)
{
    __shared__ int64_t sh8[8];
    __shared__ int sh_last;
    int64_t inc;
    if (!th_draw_inc(s, from_ctl, inc_arg, inc)) {
        return;
    }
    const int64_t p0 = (int64_t)blockIdx.x * TH_TILE + (int64_t)threadIdx.x * 4;
    int64_t n = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int64_t p = p0 + j;
        n += (p < s.N && inc >= s.th_next[p]) ? 1 : 0;
    }
    int64_t tile_total;
    cta_exclusive_scan256(n, sh8, &tile_total);
    if (threadIdx.x == 0) {
        s.th_cnt[blockIdx.x] = tile_total;
        __threadfence();
        unsigned t = atomicAdd(&s.th->ticket, 1u);
        sh_last = (t == gridDim.x - 1u) ? 1 : 0;
    }
    __syncthreads();
    if (!sh_last) {
        return;
    }
    /* last CTA: tile counts -> exclusive tile offsets (in place), the stream jumps past all draws */
    __threadfence();
    const int64_t G = gridDim.x;
    const int64_t per = (G + 255) / 256;
    const int64_t lo = (int64_t)threadIdx.x * per;
    const int64_t hi = lo + per < G ? lo + per : G;
    int64_t sum = 0;
    for (int64_t i = lo; i < hi; ++i) {
        sum += __ldcg(s.th_cnt + i);
    }
    int64_t all;
    int64_t run = cta_exclusive_scan256(sum, sh8, &all);
    for (int64_t i = lo; i < hi; ++i) {
        int64_t x = __ldcg(s.th_cnt + i);
        s.th_cnt[i] = run;
        run += x;
    }
    if (threadIdx.x == 0) {
        Thermal* th = s.th;
        uint64_t base = th->state;
        th->base = base;
        th->total = all;
        th->state = pcg_advance_inc(base, (uint64_t)all, th->inc);
        th->ticket = 0u;
    }
}

__global__ void __launch_bounds__(256) k_th_list(DevSys s, int from_ctl, int64_t inc_arg)
{
    __shared__ int64_t sh8[8];
    int64_t inc;
    if (!th_draw_inc(s, from_ctl, inc_arg, inc)) {
        return;
    }
    const int64_t p0 = (int64_t)blockIdx.x * TH_TILE + (int64_t)threadIdx.x * 4;
    bool draw[4];
    int64_t n = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int64_t p = p0 + j;
        draw[j] = p < s.N && inc >= s.th_next[p];
        n += draw[j] ? 1 : 0;
    }
    int64_t tile_total;
    int64_t k = s.th_cnt[blockIdx.x] + cta_exclusive_scan256(n, sh8, &tile_total);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (draw[j]) {
            s.th_list[k++] = (int32_t)(p0 + j);
        }
    }
}

/* One thread per draw: entry k of the list takes output k of the stream after the old state. */
__global__ void __launch_bounds__(128) k_th_eval(DevSys s, int from_ctl, int64_t inc_arg)
{
    int64_t inc;
    if (!th_draw_inc(s, from_ctl, inc_arg, inc)) {
        return;
    }
    const int64_t total = s.th->total;
    const uint64_t base = s.th->base, sinc = s.th->inc;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = s.th_list[k];
        const uint32_t u32 = pcg_output(pcg_advance_inc(base, (uint64_t)k, sinc));
        const double r = FQ_MUL((double)u32, 0x1p-32);
        const double z = fq_erfinv(FQ_SUB(FQ_MUL(2.0, r), 1.0));
        s.f_th[p] = FQ_ADD(s.th_mean, FQ_MUL(s.th_sc, z));
        s.th_next[p] += s.th_dinc[p];
    }
}

/* CTAs of k_th_eval (72 registers, 128 threads): 4 per SM, 78 k draws per pass, grid-stride beyond */
constexpr unsigned TH_EVAL_CTAS = 4 * 152;

cudaError_t launch_thermal_draw(const DevSys& s, int from_ctl, int64_t inc, cudaStream_t st)
{
    unsigned G = (unsigned)((s.N + TH_TILE - 1) / TH_TILE);
    void* args[] = {(void*)&s, (void*)&from_ctl, (void*)&inc};
    cudaError_t e = cudaLaunchKernel((void*)k_th_count, dim3(G), dim3(256), args, 0, st);
    if (e == cudaSuccess) {
        e = cudaLaunchKernel((void*)k_th_list, dim3(G), dim3(256), args, 0, st);
    }
    if (e == cudaSuccess) {
        e = cudaLaunchKernel((void*)k_th_eval, dim3(TH_EVAL_CTAS), dim3(128), args, 0, st);
    }
    return e;
}

int64_t thermal_tiles(int64_t N)
{
    return (N + TH_TILE - 1) / TH_TILE;
}

/* ------------------------------------------------------------- long-range interactions */

/*
 * Line1d System_Cuspy_LongRange (Line1d.h:617-675): every particle interacts with all others,
 * f_int(p) = sum over i != p, in index order, of (u'(i) - u'(p)) k / d^(alpha+1), d the ring distance
 * (LongRange1d::force, detail.h:844-866).  All new positions are needed before any interaction, so
 * the step is two launches: k_lr_position writes u' for all particles; k_lr_step (same pass-1 / redo
 * roles and epilogue as k_step_line) reads the new positions through shared-memory tiles, keeps each
 * particle's sum in the reference's sequential order, and does wells, forces, velocity updates and
 * the residual.
 */
__global__ void __launch_bounds__(256) k_lr_position(DevSys s)
{
    __shared__ StepShared sh;
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const int cur = sh.cur;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < s.N) {
        s.u[cur ^ 1][p] = u_next(s, s.u[cur], s.v[cur], s.a[cur], p);
    }
}

template <int POT, int PPT>
__global__ void __launch_bounds__(256) k_lr_step(DevSys s, int redo)
{
    constexpr int LR_TILE = 1024;
    __shared__ StepShared sh;
    __shared__ double tile[LR_TILE];
    if (!step_prologue(s, sh, true)) {
        return;
    }
    if (redo) {
        if (!s.cta_pending[blockIdx.x]) {
            return;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s.cta_pending[blockIdx.x] = 0;
        }
    }
    const int cur = sh.cur;
    const bool act = (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (sh.flags & RF_RESID) != 0;
    const double uf = sh.uf;
    const int64_t N = s.N;
    const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * PPT;
    const double* un = s.u[cur ^ 1];
    double up[PPT], fi[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        up[j] = p0 + j < N ? un[p0 + j] : 0.0;
        fi[j] = 0.0;
    }
    for (int64_t t0 = 0; t0 < N; t0 += LR_TILE) {
        const int cnt = (int)(N - t0 < LR_TILE ? N - t0 : LR_TILE);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            tile[k] = un[t0 + k];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            const int64_t p = p0 + j;
            if (p >= N) {
                continue;
            }
            double acc = fi[j];
            for (int k = 0; k < cnt; ++k) {
                const int64_t i = t0 + k;
                if (i == p) {
                    continue;
                }
                int64_t d = i > p ? i - p : p - i;
                if (d > s.lr_m) {
                    d = N - d;
                }
                acc = FQ_ADD(acc, FQ_MUL(FQ_SUB(tile[k], up[j]), __ldg(s.lr_pref + d)));
            }
            fi[j] = acc;
        }
    }
    double rf = 0.0, rff = 0.0;
    bool nan = false, pending = false;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const int64_t p = p0 + j;
        if (p >= N) {
            continue;
        }
        bool regen;
        double4_32a w = well_of(s, p, up[j], act, sh, regen);
        pending |= regen;
        double ff;
        double sfp = frame_pot<POT>(s, w, up[j], uf, ff);
        double sfi = FQ_ADD(sfp, fi[j]);
        double vo, ao, f;
        verlet_velocity(s, sfi, s.v[cur][p], s.a[cur][p], vo, ao, f);
        s.v[cur ^ 1][p] = vo;
        s.a[cur ^ 1][p] = ao;
        nan |= is_nan_bits(up[j]);
        if (resid) {
            double f2 = fq_smul(f, f), ff2 = fq_smul(ff, ff);
            if (j == 0) {
                rf = f2;
                rff = ff2;
            }
            else {
                rf = add_nospec(rf, f2);
                rff = add_nospec(rff, ff2);
            }
        }
    }
    if (nan) {
        sh.nan = 1;
    }
    if (pending && !redo) {
        sh.pending = 1;
        for (int j = 0; j < PPT; ++j) {
            const int64_t p = p0 + j;
            if (p < N) {
                double4_32a w = s.wc[p];
                if (!in_well(w.x, w.y, up[j]) && !non_finite(up[j])) {
                    int k = atomicAdd(&s.ctl->n_regen, 1);
                    s.regen_list[k] = (int32_t)p;
                }
            }
        }
    }
    if (pending && redo) {
        atomicOr(&s.ctl->walk_flag, 1);
    }
    step_epilogue(s, sh, redo ? EPI_REDO : EPI_LINE, rf, rff);
}

/* ------------------------------------------------------------- no-passing minimiser */

/*
 * minimise of System_Cuspy_Laplace_Nopassing (detail.h:1694-1753, class Line1d.h:173-238): one Jacobi
 * sweep per loop iteration, in the same run graph form as the dynamics (WHILE node, stop test on the
 * device).  k_nopass_update: from the previous sweep's positions (buffer cur, the reference's v_n
 * snapshot) each particle takes
 *     u = ((k (u[p-1] + u[p+1]) + k_frame u_frame) + mu umin) / ((2 k + k_frame) + mu),
 * umin the centre of its current well; the chunk is aligned at u (moving the window when needed) and,
 * while the local chunk index changes, u is recomputed with the new well.  Writes u (buffer cur ^ 1),
 * f_frame and f_potential.  k_nopass_force: f_interactions of the new positions,
 * f = (f_potential + f_interactions) + f_frame, the residual subtrees; the last CTA runs the StopList
 * test (finalize_step with RF_NOINC: no time passes).
 */
__global__ void __launch_bounds__(256) k_nopass_update(DevSys s, NopassArgs A)
{
    __shared__ StepShared sh;
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const int cur = sh.cur;
    const double uf = sh.uf;
    const int64_t N = s.N;
    const double* u0 = s.u[cur];
    const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * A.ppt;
    for (int j = 0; j < A.ppt; ++j) {
        const int64_t p = p0 + j;
        if (p >= N) {
            break;
        }
        const double uneigh = p == 0       ? FQ_ADD(u0[N - 1], u0[1])
                              : p == N - 1 ? FQ_ADD(u0[N - 2], u0[0])
                                           : FQ_ADD(u0[p - 1], u0[p + 1]);
        const double* y = s.data + p * s.W;
        int64_t i = s.cidx[p];
        double umin = 0.0, u = 0.0;
        for (int it = 0;; ++it) {
            if (it >= NOPASS_MAX_REALIGN) {
                atomicOr(&s.ctl->walk_flag, 1); /* reported as an error by the finalisation */
                break;
            }
            umin = FQ_MUL(0.5, FQ_ADD(y[i], y[i + 1]));
            u = FQ_DIV(FQ_ADD(FQ_ADD(FQ_MUL(s.k, uneigh), FQ_MUL(s.k_frame, uf)), FQ_MUL(s.mu, umin)), A.den);
            dev_align(s, p, u);
            const int64_t jj = s.cidx[p];
            if (jj == i) {
                break;
            }
            i = jj;
        }
        s.u[cur ^ 1][p] = u;
        s.v[cur ^ 1][p] = s.v[cur][p];
        s.a[cur ^ 1][p] = s.a[cur][p];
        A.f_frame[p] = FQ_MUL(s.k_frame, FQ_SUB(uf, u));
        A.f_pot[p] = FQ_MUL(s.mu, FQ_SUB(umin, u));
    }
}

__global__ void __launch_bounds__(256) k_nopass_force(DevSys s, NopassArgs A)
{
    __shared__ StepShared sh;
    if (!step_prologue(s, sh, true)) {
        return;
    }
    const int cur = sh.cur;
    const int64_t N = s.N;
    const double* u1 = s.u[cur ^ 1];
    const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * A.ppt;
    double rf = 0.0, rff = 0.0;
    for (int j = 0; j < A.ppt; ++j) {
        const int64_t p = p0 + j;
        if (p >= N) {
            break;
        }
        const double u = u1[p];
        const double uL = u1[p == 0 ? N - 1 : p - 1], uR = u1[p == N - 1 ? 0 : p + 1];
        const double fi = scale(FQ_ADD(FQ_SUB(uL, scale_pow2(u, 1, 2.0)), uR), s.s_k);
        const double ff = A.f_frame[p];
        const double f = FQ_ADD(FQ_ADD(A.f_pot[p], fi), ff);
        A.f_int[p] = fi;
        A.f[p] = f;
        const double f2 = FQ_MUL(f, f), ff2 = FQ_MUL(ff, ff);
        if (j == 0) {
            rf = f2;
            rff = ff2;
        }
        else {
            rf = FQ_ADD(rf, f2);
            rff = FQ_ADD(rff, ff2);
        }
    }
    step_epilogue(s, sh, EPI_LINE, rf, rff);
}

cudaError_t launch_nopass_iteration(const DevSys& s, const LineGeom& g, const NopassArgs& A, cudaStream_t st)
{
    k_nopass_update<<<(unsigned)g.grid, (unsigned)g.threads, 0, st>>>(s, A);
    k_nopass_force<<<(unsigned)g.grid, (unsigned)g.threads, 0, st>>>(s, A);
    return cudaGetLastError();
}

/* ------------------------------------------------------------- small systems: one cluster */

/*
 * A whole run of a small Line1d / Particles system in one launch of one thread-block cluster (up to
 * 16 CTAs on 16 SMs).  For small N the graph path is bound by its per-step launch and node overhead
 * (about 18 us per time step at N = 1024, no faster than one CPU core); here the state stays in
 * registers for the whole run, the new positions at tile edges cross CTA boundaries through
 * distributed shared memory, and one cluster barrier per time step replaces the per-step launches.
 *
 * Every CTA has its particle threads and one control warp (the last warp).  Time step t:
 *   position update -> cluster barrier A_t -> wells, forces, velocities, the CTA's residual subtree
 *   and counters, published to CTA 0's slot t % 2 -> position update of step t + 1 -> A_{t+1} ...
 * Meanwhile, after A_{t+1}, CTA 0's control warp sums step t's subtrees, applies its counters and
 * runs the same stop tests as the graph path (finalize_ctl); its decision is read by every thread
 * after A_{t+2}.  The decision thus comes two barriers late: when it says stop after step t, the
 * threads have already taken step t + 1, and they restore the state from before that step (positions,
 * velocities, accelerations, and the well and chunk window as they were) -- the step's counters were
 * never applied.  The stop tests therefore leave the critical path, and one barrier per step remains.
 * Arithmetic, the residual tree (aligned power-of-two tiles) and the stop tests are those of
 * k_step_line, and chunk windows move as k_regen moves them, so the results equal the graph path's
 * bit for bit.  Runs that record a trajectory (adjoint) use the graph path.
 */

/* Named barrier 1 over the particle threads of the CTA (the control warp is not in it). */
__device__ __forceinline__ void particle_bar(int n)
{
    asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
}

/* particle_bar that also returns whether any particle thread passed a non-zero flag */
__device__ __forceinline__ int particle_bar_or(int n, int flag)
{
    int r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.or.pred q, 1, %2, p;\n\t"
                 "selp.s32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"(flag), "r"(n)
                 : "memory");
    return r;
}

/* cta_tree2 over the first nt threads of the CTA (nt a multiple of 32), with the named barrier */
__device__ __forceinline__ double2 particle_tree2(double x, double y, double* sh, int nt)
{
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        double xo = __shfl_down_sync(0xffffffffu, x, m);
        double yo = __shfl_down_sync(0xffffffffu, y, m);
        if ((threadIdx.x & (2 * m - 1)) == 0) {
            x = add_nospec(x, xo);
            y = add_nospec(y, yo);
        }
    }
    int nw = nt >> 5;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    particle_bar(nt);
    if (lane == 0) {
        sh[wid] = x;
        sh[32 + wid] = y;
    }
    particle_bar(nt);
    if (wid == 0) {
        double a = lane < nw ? sh[lane] : 0.0;
        double b = lane < nw ? sh[32 + lane] : 0.0;
#pragma unroll
        for (int m = 1; m < 32; m <<= 1) {
            double ao = __shfl_down_sync(0xffffffffu, a, m);
            double bo = __shfl_down_sync(0xffffffffu, b, m);
            if ((threadIdx.x & (2 * m - 1)) == 0) {
                a = add_nospec(a, ao);
                b = add_nospec(b, bo);
            }
        }
        x = a;
        y = b;
    }
    return make_double2(x, y);
}

template <int POT, int INTER, int PPT>
__global__ void __launch_bounds__(SMALL_THREADS_MAX + 32, 1) k_run_small(DevSys s)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ double sh_un[2][SMALL_THREADS_MAX * PPT];
    __shared__ double red[64];
    /* CTA 0 keeps the run-control block and the StopList window, and per step parity the CTAs'
     * residual subtrees and counters, and the stop decision */
    __shared__ Ctl sc;
    __shared__ double sring[SMALL_RING_MAX];
    __shared__ double2 spart[2][SMALL_MAX_CTAS];
    __shared__ unsigned long long sl_ds[2], sl_da[2];
    __shared__ int sl_nan[2], sl_walk[2], sl_stop[2];
    /* this CTA's counters of the current step */
    __shared__ int sh_nan, sh_walk;
    __shared__ unsigned long long sh_ds, sh_da;
    /* window moves of this step shared by the CTA's particle threads (fwd_move_*) */
    constexpr int SMALL_MOVES = 64;
    __shared__ FwdMove sh_moves[SMALL_MOVES];
    __shared__ int sh_nmove;

    const unsigned rank = cluster.block_rank();
    const unsigned G = cluster.num_blocks();
    const int tid = threadIdx.x;
    const int pt = (int)blockDim.x - 32; /* particle threads; the last warp is the control warp */
    const bool ctrl = tid >= pt;
    const int64_t N = s.N;
    const int64_t tile = (int64_t)pt * PPT;
    const int64_t base = (int64_t)rank * tile;
    const int64_t p0 = base + (int64_t)tid * PPT;
    const Ctl* gc = s.ctl;
    const int flags = gc->flags;
    const bool act = (flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (flags & RF_RESID) != 0;
    const double vdt = gc->vdt;
    double uf = gc->u_frame;
    int cur = gc->cur;
    const int64_t nring = (resid && gc->niter_tol > 0) ? gc->niter_tol : 0;
    if (rank == 0) {
        if (tid == 0) {
            sc = *gc;
        }
        for (int64_t i = tid; i < nring; i += blockDim.x) {
            sring[i] = s.ring[i];
        }
        if (tid < 2) {
            sl_ds[tid] = 0ull;
            sl_da[tid] = 0ull;
            sl_nan[tid] = 0;
            sl_walk[tid] = 0;
            sl_stop[tid] = 0;
        }
    }

    /* ring neighbours of the tile's first and last particle: (CTA rank, index in its tile) */
    const int64_t plast = (base + tile < N ? base + tile : N) - 1;
    const int64_t pl = base == 0 ? N - 1 : base - 1;
    const int64_t pr = plast + 1 == N ? 0 : plast + 1;
    const int il = (int)(pl % tile), ir = (int)(pr % tile);
    const double* left[2] = {cluster.map_shared_rank(&sh_un[0][0], (unsigned)(pl / tile)),
                             cluster.map_shared_rank(&sh_un[1][0], (unsigned)(pl / tile))};
    const double* right[2] = {cluster.map_shared_rank(&sh_un[0][0], (unsigned)(pr / tile)),
                              cluster.map_shared_rank(&sh_un[1][0], (unsigned)(pr / tile))};
    Ctl* sc0 = cluster.map_shared_rank(&sc, 0);
    double2* spart0 = cluster.map_shared_rank(&spart[0][0], 0);
    unsigned long long* sl_ds0 = cluster.map_shared_rank(&sl_ds[0], 0);
    unsigned long long* sl_da0 = cluster.map_shared_rank(&sl_da[0], 0);
    int* sl_nan0 = cluster.map_shared_rank(&sl_nan[0], 0);
    int* sl_walk0 = cluster.map_shared_rank(&sl_walk[0], 0);
    const int* sl_stop0 = cluster.map_shared_rank(&sl_stop[0], 0);

    double u[PPT], v[PPT], a[PPT];
    double4_32a w[PPT];
    /* the state before the latest step, kept for the rollback of a step taken after the stop */
    double pu[PPT], pv[PPT], pa[PPT];
    int64_t pstart[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        int64_t p = p0 + j;
        if (!ctrl && p < N) {
            u[j] = s.u[cur][p];
            v[j] = s.v[cur][p];
            a[j] = s.a[cur][p];
            w[j] = s.wc[p];
        }
        else {
            u[j] = v[j] = a[j] = 0.0;
            w[j] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
        }
        pu[j] = u[j];
        pv[j] = v[j];
        pa[j] = a[j];
        pstart[j] = 0;
    }
    /* one particle per thread: latency bound, all fp64 on the fp64 pipe; more: throughput bound, split */
    constexpr unsigned SOFT = PPT >= 2 ? STEP_SOFT : 0u;
    /* pcg32 stride of pt steps, x -> mv_a x + mv_c, for the shared draws of window moves */
    const uint64_t mv_c = pcg_advance(0ULL, (uint64_t)pt);
    const uint64_t mv_a = pcg_advance(1ULL, (uint64_t)pt) - mv_c;
    int buf = 0;
    double uf_prev = uf;
    for (int64_t t = 0;; ++t) {
        const double uf_t = (flags & RF_FLOW) ? FQ_ADD(uf, vdt) : uf;
        double un[PPT];
        if (!ctrl) {
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                un[j] = S_ADD(3, S_ADD(2, u[j], S_MUL(0, s.dt, v[j])), S_MUL(1, s.hdt2, a[j]));
                sh_un[buf][tid * PPT + j] = un[j];
            }
        }
        if (tid == 0) {
            sh_ds = 0ull;
            sh_da = 0ull;
            sh_nan = 0;
            sh_walk = 0;
            sh_nmove = 0;
        }
        /* A_t: every tile's new positions, the subtrees and counters of step t - 1, and the decision
         * after step t - 2 (slot t % 2) */
        cluster.sync();
        if (t >= 2 && sl_stop0[t & 1]) {
            /* stopped after step t - 2: restore the state before step t - 1 */
            if (!ctrl) {
#pragma unroll
                for (int j = 0; j < PPT; ++j) {
                    int64_t p = p0 + j;
                    u[j] = pu[j];
                    v[j] = pv[j];
                    a[j] = pa[j];
                    if (p >= N) {
                        continue;
                    }
                    bool placed = false;
                    if (s.start[p] != pstart[j]) {
                        /* the window moved in the step taken after the stop: put it back */
                        double acc;
                        seq_fill(s, p, pstart[j], s.W, s.data + p * s.W, &acc);
                        s.start[p] = pstart[j];
                        s.acc_end[p] = acc;
                        placed = true;
                    }
                    /* the well of the restored position (index, cached well) in the restored window */
                    double4_32a ww = s.wc[p];
                    if ((placed || !in_well(ww.x, ww.y, u[j])) && !non_finite(u[j]) &&
                        !window_search(s, p, u[j], ww)) {
                        dev_align(s, p, u[j]);
                    }
                }
            }
            break;
        }
        const double uf_last = uf_prev; /* u_frame of step t - 1, for its stop tests */
        uf_prev = uf_t;
        uf = uf_t;
        if (ctrl) {
            if (rank == 0 && t >= 1) {
                /* the decision after step t - 1 */
                const int q = (int)((t - 1) & 1);
                const int lane = tid - pt;
                double tx = 0.0, ty = 0.0;
                if (resid) {
                    /* the canonical tree over the CTA subtrees, zero padded (as tree_partials): G <= 32 */
                    double x = 0.0, y = 0.0;
                    if ((unsigned)lane < G) {
                        x = spart[q][lane].x;
                        y = spart[q][lane].y;
                    }
                    tx = warp_tree(x);
                    ty = warp_tree(y);
                }
                if (lane == 0) {
                    sc.s_sum = (long long)((unsigned long long)sc.s_sum + sl_ds[q]);
                    sc.a_count = (long long)((unsigned long long)sc.a_count + sl_da[q]);
                    if (sl_nan[q]) {
                        sc.nan_flag = 1;
                    }
                    if (sl_walk[q]) {
                        sc.walk_flag = 1;
                    }
                    sl_ds[q] = 0ull;
                    sl_da[q] = 0ull;
                    sl_nan[q] = 0;
                    sl_walk[q] = 0;
                    finalize_ctl(&sc, sring, uf_last, tx, ty);
                    sl_stop[q] = (sc.done || sc.error || (globaltimer() - sc.launch_t0) >= sc.budget_ns) ? 1 : 0;
                }
            }
            buf ^= 1;
            continue;
        }
        /* the particle threads take step t */
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            pu[j] = u[j];
            pv[j] = v[j];
            pa[j] = a[j];
            if (p0 + j < N) {
                pstart[j] = s.start[p0 + j];
            }
        }
        double rf = 0.0, rff = 0.0;
        bool nan = false;
        /* plastic activity of a particle whose well index went from gold to gnew */
        auto count_move = [&](int64_t p, int64_t gold, int64_t gnew) {
            if (act && gnew != gold) {
                int64_t ref = s.i_n[p];
                long long ds = absll(gnew - ref) - absll(gold - ref);
                long long da = (long long)(gnew != ref) - (long long)(gold != ref);
                atomicAdd(&sh_ds, (unsigned long long)ds);
                atomicAdd(&sh_da, (unsigned long long)da);
            }
        };
        /* wells: a search inside the chunk window, or a window move */
        int64_t gold[PPT];
        bool mv[PPT];
        bool any_mv = false;
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            int64_t p = p0 + j;
            mv[j] = false;
            if (p >= N) {
                continue;
            }
            double up = un[j];
            double4_32a ww = w[j];
            if (!in_well(ww.x, ww.y, up) && !non_finite(up)) {
                gold[j] = s.gidx[p];
                if (window_search(s, p, up, ww)) {
                    count_move(p, gold[j], s.gidx[p]);
                    w[j] = ww;
                }
                else {
                    mv[j] = true;
                    any_mv = true;
                }
            }
        }
        if (particle_bar_or(pt, any_mv ? 1 : 0)) {
            /* moves planned here are drawn by all particle threads of the CTA, then summed by their
             * owners; the others (more than SMALL_MOVES, or not a forward move) go through dev_align */
            int slot[PPT];
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                slot[j] = -1;
                if (mv[j]) {
                    int k = atomicAdd(&sh_nmove, 1);
                    if (k < SMALL_MOVES) {
                        FwdMove m;
                        const bool ready = next_window_ready(s, p0 + j);
                        if (fwd_move_plan(s, p0 + j, un[j], m)) {
                            m.next = ready ? 1 : 0;
                            sh_moves[k] = m;
                            slot[j] = k;
                        }
                        else {
                            sh_moves[k].p = -1;
                        }
                    }
                }
            }
            if (tid == 0) {
                /* the moved windows' next-window buffers are out of date after this run */
                atomicOr(&sc0->nx_stale, 1);
            }
            particle_bar(pt);
            const int nm = sh_nmove < SMALL_MOVES ? sh_nmove : SMALL_MOVES;
            for (int k = 0; k < nm; ++k) {
                if (sh_moves[k].p >= 0) {
                    if (sh_moves[k].next) {
                        fwd_move_copy(s, sh_moves[k], tid, pt);
                    }
                    else {
                        fwd_move_draws(s, sh_moves[k], tid, pt, mv_a, mv_c);
                    }
                }
            }
            particle_bar(pt);
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                if (!mv[j]) {
                    continue;
                }
                int64_t p = p0 + j;
                if (slot[j] >= 0) {
                    if (sh_moves[slot[j]].next) {
                        fwd_move_finish(s, sh_moves[slot[j]]);
                    }
                    else {
                        fwd_move_sum(s, sh_moves[slot[j]]);
                    }
                }
                else {
                    dev_align(s, p, un[j]); /* moves the chunk window; a failed search sets walk_flag */
                    if (((volatile Ctl*)s.ctl)->walk_flag) {
                        sh_walk = 1;
                    }
                }
                w[j] = s.wc[p];
                count_move(p, gold[j], s.gidx[p]);
            }
        }
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            int64_t p = p0 + j;
            if (p >= N) {
                continue;
            }
            double up = un[j];
            const double4_32a ww = w[j];
            double ff;
            double sfp = frame_pot<POT, SOFT>(s, ww, up, uf, ff);
            double fi = 0.0;
            if (inter_ring(INTER)) {
                int li = tid * PPT + j;
                double uL = li > 0 ? sh_un[buf][li - 1] : left[buf][il];
                double uR = (li + 1 < tile && p + 1 < N) ? sh_un[buf][li + 1] : right[buf][ir];
                fi = ring_force<INTER, SOFT>(s, uL, up, uR);
            }
            double sfi = S_ADD(9, sfp, fi);
            double vn, an, f;
            verlet_velocity<SOFT>(s, sfi, v[j], a[j], vn, an, f);
            u[j] = up;
            v[j] = vn;
            a[j] = an;
            nan |= is_nan_bits(up);
            if (resid) {
                double f2 = mul_nospec(f, f), ff2 = mul_nospec(ff, ff);
                if (j == 0) {
                    rf = f2;
                    rff = ff2;
                }
                else {
                    rf = add_nospec(rf, f2);
                    rff = add_nospec(rff, ff2);
                }
            }
        }
        if (nan) {
            sh_nan = 1;
        }
        double2 sfs = make_double2(0.0, 0.0);
        if (resid) {
            sfs = particle_tree2(rf, rff, red, pt);
        }
        particle_bar(pt);
        if (tid == 0) {
            /* publish step t to CTA 0's slot t % 2 */
            const int q = (int)(t & 1);
            if (resid) {
                spart0[q * SMALL_MAX_CTAS + rank] = sfs;
            }
            if (sh_ds) {
                atomicAdd(sl_ds0 + q, sh_ds);
            }
            if (sh_da) {
                atomicAdd(sl_da0 + q, sh_da);
            }
            if (sh_nan) {
                atomicOr(sl_nan0 + q, 1);
            }
            if (sh_walk) {
                atomicOr(sl_walk0 + q, 1);
            }
        }
        buf ^= 1;
    }
    cur = sc0->cur;
    if (!ctrl) {
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            int64_t p = p0 + j;
            if (p < N) {
                s.u[cur][p] = u[j];
                s.v[cur][p] = v[j];
                s.a[cur][p] = a[j];
            }
        }
    }
    if (rank == 0) {
        for (int64_t i = tid; i < nring; i += blockDim.x) {
            s.ring[i] = sring[i];
        }
        if (tid == 0) {
            *s.ctl = sc;
        }
    }
    /* no CTA may exit while others still read its shared memory */
    cluster.sync();
}

SmallGeom small_geometry(int64_t N, int max_ctas)
{
    SmallGeom g;
    int64_t per = (N + max_ctas - 1) / max_ctas;
    int64_t tile = 32;
    while (tile < per) {
        tile <<= 1;
    }
    g.threads = (int)(tile < 256 ? tile : 256);
    g.ppt = (int)(tile / g.threads);
    g.ctas = (int)((N + tile - 1) / tile);
    g.ok = N >= 1 && tile <= 1024 && max_ctas <= SMALL_MAX_CTAS;
    return g;
}

template <int POT, int INTER>
static const void* small_kernel_t(int ppt)
{
    switch (ppt) {
        case 1: return (const void*)k_run_small<POT, INTER, 1>;
        case 2: return (const void*)k_run_small<POT, INTER, 2>;
        default: return (const void*)k_run_small<POT, INTER, 4>;
    }
}

static const void* small_kernel(const DevSys& s, const SmallGeom& g)
{
    /* the Quartic interactions exist with the Cuspy potential only (Line1d.h:428, :562) */
    if (s.inter == INTER_QUARTIC1D) {
        return small_kernel_t<POT_CUSPY, INTER_QUARTIC1D>(g.ppt);
    }
    if (s.inter == INTER_QUARTICGRAD1D) {
        return small_kernel_t<POT_CUSPY, INTER_QUARTICGRAD1D>(g.ppt);
    }
    if (s.inter == INTER_LAPLACE1D) {
        return s.pot == POT_CUSPY ? small_kernel_t<POT_CUSPY, INTER_LAPLACE1D>(g.ppt)
               : s.pot == POT_SEMISMOOTH ? small_kernel_t<POT_SEMISMOOTH, INTER_LAPLACE1D>(g.ppt)
                                         : small_kernel_t<POT_SMOOTH, INTER_LAPLACE1D>(g.ppt);
    }
    return s.pot == POT_CUSPY ? small_kernel_t<POT_CUSPY, INTER_NONE>(g.ppt)
           : s.pot == POT_SEMISMOOTH ? small_kernel_t<POT_SEMISMOOTH, INTER_NONE>(g.ppt)
                                     : small_kernel_t<POT_SMOOTH, INTER_NONE>(g.ppt);
}

static void small_launch_config(const SmallGeom& g, cudaStream_t st, cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr)
{
    cfg = {};
    cfg.gridDim = dim3((unsigned)g.ctas);
    cfg.blockDim = dim3((unsigned)g.threads + 32u); /* particle threads and the control warp */
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)g.ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
}

bool small_cluster_fits(const DevSys& s, const SmallGeom& g)
{
    const void* f = small_kernel(s, g);
    if (cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    small_launch_config(g, nullptr, cfg, attr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, f, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n >= 1;
}

cudaError_t launch_small_run(const DevSys& s, const SmallGeom& g, cudaStream_t st)
{
    const void* f = small_kernel(s, g);
    if (g.ctas > 8) {
        /* clusters above the portable size of 8 must be allowed per kernel */
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) {
            return e;
        }
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    small_launch_config(g, st, cfg, attr);
    DevSys arg = s;
    arg.in_graph = 0; /* not inside the run graph: no conditional handles to set */
    void* args[] = {(void*)&arg};
    return cudaLaunchKernelExC(&cfg, f, args);
}

/* ------------------------------------------------------------- geometry */

LineGeom line_geometry(int64_t N)
{
    LineGeom g;
    /* enough CTAs to fill 152 SMs when N allows, power-of-two tiles for the canonical reduction */
    int64_t tile = 512;
    while (tile > 32 && (N + tile - 1) / tile < 2 * 152) {
        tile >>= 1;
    }
    g.ppt = tile >= 512 ? 2 : 1;
    g.threads = (int)(tile / g.ppt);
    g.grid = (N + tile - 1) / tile;
    return g;
}

int64_t grid_reduce_ctas(int64_t N)
{
    return (N + 1023) / 1024;
}

int64_t step_ctas(const DevSys& s, const LineGeom& g)
{
    if (inter_grid(s.inter)) {
        return ((s.cols + 31) / 32) * ((s.rows + grid_tile_rows(s) - 1) / grid_tile_rows(s));
    }
    return g.grid;
}

/* ------------------------------------------------------------- run graph */

template <int POT, int INTER, bool TH = false, int MODE = KMODE_GENERAL>
static void* line_kernel_t(int ppt)
{
    return ppt == 2 ? (void*)k_step_line<POT, INTER, 2, STEP_SOFT, TH, MODE>
                    : (void*)k_step_line<POT, INTER, 1, STEP_SOFT, TH, MODE>;
}

template <int MODE>
static void* special_kernel(const DevSys& s, const LineGeom& g)
{
    if (s.inter == INTER_LAPLACE1D) {
        switch (s.pot) {
            case POT_CUSPY: return line_kernel_t<POT_CUSPY, INTER_LAPLACE1D, false, MODE>(g.ppt);
            case POT_SEMISMOOTH: return line_kernel_t<POT_SEMISMOOTH, INTER_LAPLACE1D, false, MODE>(g.ppt);
            default: return line_kernel_t<POT_SMOOTH, INTER_LAPLACE1D, false, MODE>(g.ppt);
        }
    }
    switch (s.pot) {
        case POT_CUSPY: return line_kernel_t<POT_CUSPY, INTER_NONE, false, MODE>(g.ppt);
        case POT_SEMISMOOTH: return line_kernel_t<POT_SEMISMOOTH, INTER_NONE, false, MODE>(g.ppt);
        default: return line_kernel_t<POT_SMOOTH, INTER_NONE, false, MODE>(g.ppt);
    }
}

bool plain_runs_apply(const DevSys& s)
{
    return !s.f_th && (s.inter == INTER_LAPLACE1D || s.inter == INTER_NONE);
}

static void* step_kernel(const DevSys& s, const LineGeom& g, int mode = KMODE_GENERAL)
{
    if (mode != KMODE_GENERAL && plain_runs_apply(s)) {
        return mode == KMODE_PLAIN ? special_kernel<KMODE_PLAIN>(s, g) : special_kernel<KMODE_RESID>(s, g);
    }
    if (s.f_th) {
        /* RandomNormalForcing systems: Cuspy with Laplace1d, Quartic1d or no interactions */
        switch (s.inter) {
            case INTER_LAPLACE1D: return line_kernel_t<POT_CUSPY, INTER_LAPLACE1D, true>(g.ppt);
            case INTER_QUARTIC1D: return line_kernel_t<POT_CUSPY, INTER_QUARTIC1D, true>(g.ppt);
            default: return line_kernel_t<POT_CUSPY, INTER_NONE, true>(g.ppt);
        }
    }
    if (s.inter == INTER_LONGRANGE1D) {
        return g.ppt == 2 ? (void*)k_lr_step<POT_CUSPY, 2> : (void*)k_lr_step<POT_CUSPY, 1>;
    }
    if (s.inter == INTER_QUARTICGRAD2D) {
        return (void*)k_step_grid<POT_CUSPY, INTER_QUARTICGRAD2D>;
    }
    if (s.inter == INTER_QUARTIC1D) {
        return line_kernel_t<POT_CUSPY, INTER_QUARTIC1D>(g.ppt);
    }
    if (s.inter == INTER_QUARTICGRAD1D) {
        return line_kernel_t<POT_CUSPY, INTER_QUARTICGRAD1D>(g.ppt);
    }
    if (s.inter == INTER_LAPLACE2D) {
        switch (s.pot) {
            case POT_CUSPY: return (void*)k_step_grid2<POT_CUSPY>;
            case POT_SEMISMOOTH: return (void*)k_step_grid2<POT_SEMISMOOTH>;
            default: return (void*)k_step_grid2<POT_SMOOTH>;
        }
    }
    if (s.inter == INTER_LAPLACE1D) {
        switch (s.pot) {
            case POT_CUSPY: return line_kernel_t<POT_CUSPY, INTER_LAPLACE1D>(g.ppt);
            case POT_SEMISMOOTH: return line_kernel_t<POT_SEMISMOOTH, INTER_LAPLACE1D>(g.ppt);
            default: return line_kernel_t<POT_SMOOTH, INTER_LAPLACE1D>(g.ppt);
        }
    }
    switch (s.pot) {
        case POT_CUSPY: return line_kernel_t<POT_CUSPY, INTER_NONE>(g.ppt);
        case POT_SEMISMOOTH: return line_kernel_t<POT_SEMISMOOTH, INTER_NONE>(g.ppt);
        default: return line_kernel_t<POT_SMOOTH, INTER_NONE>(g.ppt);
    }
}

static cudaError_t add_kernel(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps,
                              void* func, dim3 grid, dim3 block, void** args)
{
    cudaKernelNodeParams kp = {};
    kp.func = func;
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    return cudaGraphAddKernelNode(node, graph, deps, ndeps, &kp);
}

static cudaError_t add_conditional(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t ndeps,
                                   cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraph_t* body)
{
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaError_t e = cudaGraphAddNode(node, graph, deps, nullptr, ndeps, &np);
    if (e == cudaSuccess) {
        *body = np.conditional.phGraph_out[0];
    }
    return e;
}

/*
 * Host-driven form of one loop iteration (no conditional nodes, e.g. for profilers that cannot
 * profile kernels inside conditional graphs): pass 1, the regeneration kernel and the redo are always
 * launched; the latter two do nothing when no CTA is pending.
 */
cudaError_t launch_iteration(const DevSys& s, const LineGeom& g0, cudaStream_t st, int mode)
{
    bool is2d = inter_grid(s.inter);
    dim3 grid, block;
    if (is2d) {
        grid = dim3((unsigned)((s.cols + 31) / 32), (unsigned)((s.rows + grid_tile_rows(s) - 1) / grid_tile_rows(s)));
        block = dim3(32, 8);
    }
    else {
        grid = dim3((unsigned)g0.grid);
        block = dim3((unsigned)g0.threads);
    }
    void* fstep = step_kernel(s, g0, mode);
    int pass1 = 0, pass2 = 1;
    void* args1[] = {(void*)&s, (void*)&pass1};
    void* args2[] = {(void*)&s, (void*)&pass2};
    void* argsr[] = {(void*)&s};
    cudaError_t e = cudaSuccess;
    if (s.f_th) {
        e = launch_thermal_draw(s, 1, 0, st);
    }
    if (e == cudaSuccess && s.inter == INTER_LONGRANGE1D) {
        e = cudaLaunchKernel((void*)k_lr_position, dim3((unsigned)((s.N + 255) / 256)), dim3(256), argsr, 0, st);
    }
    if (e == cudaSuccess) {
        e = cudaLaunchKernel(fstep, grid, block, args1, 0, st);
    }
    if (e == cudaSuccess) {
        e = cudaLaunchKernel((void*)k_regen, dim3(4 * 152), dim3(128), argsr, 0, st);
    }
    if (e == cudaSuccess) {
        e = cudaLaunchKernel(fstep, grid, block, args2, 0, st);
    }
    if (e == cudaSuccess && is2d) {
        e = cudaLaunchKernel((void*)k_reduce_grid, dim3((unsigned)grid_reduce_ctas(s.N)), dim3(256), argsr, 0, st);
    }
    return e;
}

#define GR(expr)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (expr);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            cudaGraphDestroy(g);                                                                       \
            return e_;                                                                                 \
        }                                                                                              \
    } while (0)

/*
 * The run graph: WHILE(h_while) { step pass 1 ; IF(h_if) { regenerate windows ; redo pending CTAs } ;
 * [2d: reduce + finalise] }.  `s` is updated with the two conditional handles (kernel arguments).
 */
cudaError_t build_run_graph(DevSys& s, const LineGeom& g0, cudaGraphExec_t* exec, int mode)
{
    cudaGraph_t g;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) {
        return e;
    }
    cudaGraphConditionalHandle hw, hi;
    GR(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t wnode;
    cudaGraph_t body;
    GR(add_conditional(&wnode, g, nullptr, 0, hw, cudaGraphCondTypeWhile, &body));
    GR(cudaGraphConditionalHandleCreate(&hi, body, 0, cudaGraphCondAssignDefault));
    s.h_while = hw;
    s.h_if = hi;
    s.in_graph = 1;

    bool is2d = inter_grid(s.inter);
    dim3 grid, block;
    if (is2d) {
        grid = dim3((unsigned)((s.cols + 31) / 32), (unsigned)((s.rows + grid_tile_rows(s) - 1) / grid_tile_rows(s)));
        block = dim3(32, 8);
    }
    else {
        grid = dim3((unsigned)g0.grid);
        block = dim3((unsigned)g0.threads);
    }
    void* fstep = step_kernel(s, g0, mode);
    int pass1 = 0, pass2 = 1;
    void* args1[] = {(void*)&s, (void*)&pass1};
    void* args2[] = {(void*)&s, (void*)&pass2};
    void* argsr[] = {(void*)&s};
    cudaGraphNode_t nstep, nif;
    int th_from_ctl = 1;
    int64_t th_inc = 0;
    void* argst[] = {(void*)&s, (void*)&th_from_ctl, (void*)&th_inc};
    if (s.f_th) {
        /* updated_inc of the step: thermal draws before the step's forces */
        cudaGraphNode_t ncount, nlist, neval;
        dim3 gth((unsigned)thermal_tiles(s.N));
        GR(add_kernel(&ncount, body, nullptr, 0, (void*)k_th_count, gth, dim3(256), argst));
        GR(add_kernel(&nlist, body, &ncount, 1, (void*)k_th_list, gth, dim3(256), argst));
        GR(add_kernel(&neval, body, &nlist, 1, (void*)k_th_eval, dim3(TH_EVAL_CTAS), dim3(128), argst));
        GR(add_kernel(&nstep, body, &neval, 1, fstep, grid, block, args1));
    }
    else if (s.inter == INTER_LONGRANGE1D) {
        /* all new positions before the all-pairs interaction */
        cudaGraphNode_t npos;
        GR(add_kernel(&npos, body, nullptr, 0, (void*)k_lr_position, dim3((unsigned)((s.N + 255) / 256)), dim3(256),
                      argsr));
        GR(add_kernel(&nstep, body, &npos, 1, fstep, grid, block, args1));
    }
    else {
        GR(add_kernel(&nstep, body, nullptr, 0, fstep, grid, block, args1));
    }
    cudaGraph_t ifbody;
    GR(add_conditional(&nif, body, &nstep, 1, hi, cudaGraphCondTypeIf, &ifbody));
    cudaGraphNode_t nregen, nredo;
    GR(add_kernel(&nregen, ifbody, nullptr, 0, (void*)k_regen, dim3(4 * 152), dim3(128), argsr));
    GR(add_kernel(&nredo, ifbody, &nregen, 1, fstep, grid, block, args2));
    if (is2d) {
        cudaGraphNode_t nred;
        GR(add_kernel(&nred, body, &nif, 1, (void*)k_reduce_grid, dim3((unsigned)grid_reduce_ctas(s.N)), dim3(256),
                      argsr));
    }
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return e;
}

/* The no-passing minimiser's graph: WHILE(h_while) { k_nopass_update ; k_nopass_force }. */
cudaError_t build_nopass_graph(const DevSys& s0, const LineGeom& g0, const NopassArgs& A, cudaGraphExec_t* exec)
{
    DevSys s = s0;
    cudaGraph_t g;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) {
        return e;
    }
    cudaGraphConditionalHandle hw;
    GR(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t wnode;
    cudaGraph_t body;
    GR(add_conditional(&wnode, g, nullptr, 0, hw, cudaGraphCondTypeWhile, &body));
    s.h_while = hw;
    s.h_if = 0;
    s.in_graph = 1;
    NopassArgs a = A;
    void* args[] = {(void*)&s, (void*)&a};
    cudaGraphNode_t nup, nforce;
    GR(add_kernel(&nup, body, nullptr, 0, (void*)k_nopass_update, dim3((unsigned)g0.grid), dim3((unsigned)g0.threads),
                  args));
    GR(add_kernel(&nforce, body, &nup, 1, (void*)k_nopass_force, dim3((unsigned)g0.grid), dim3((unsigned)g0.threads),
                  args));
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return e;
}

} // namespace fqsb
