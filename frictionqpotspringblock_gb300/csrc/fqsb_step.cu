/*
 * Fused velocity-Verlet step kernels (sm_103a, FP64).
 *
 * One launch = one System::timeStep (include/FrictionQPotSpringBlock/detail.h:1539-1570)
 * over all particles, fused with everything timeStep calls:
 *   u update (:1549), updated_u -> potential force with the well search
 *   (Cuspy::force :139-170 / SemiSmooth :236-277 / Smooth :379-409), interaction
 *   (Laplace1d::force :474-487 / Laplace2d::force :545-583), frame force (:1353-1356),
 *   three velocity updates with damping and force sums (:1552-1565, :1321-1395),
 *   the NaN check (:1567-1569),
 * and, when the run asks for it, with the residual terms of minimise / timeStepsUntilEvent
 * (residual :1512-1520, StopList test :1780-1783) and the plastic-activity bookkeeping
 * (:1768-1778, :1855-1866).  The last CTA to finish a step evaluates the step's stop tests on
 * the device, so a multi-step run needs no host synchronisation per step.
 *
 * State is double buffered (u, v, a)[cur] -> (u, v, a)[cur ^ 1]; neighbours' updated positions
 * come from shared memory inside a CTA and are recomputed from the old state at CTA edges.
 * Only a particle that leaves its current well touches its chunk row (dev_align).
 *
 * Arithmetic uses explicit __dadd_rn / __dmul_rn in the reference's order (no fma contraction),
 * so results equal the CPU oracle bit for bit.  Algebraically neutral shortcuts only:
 * the partial sum f_frame + f_potential + f_interactions is formed once per step (it is the same
 * in every computeForce of the step), and multiplications by parameters that are exactly 1.0
 * are skipped (x * 1.0 == x) in the UNITS instantiation.
 */
#include "fqsb_internal.h"

namespace fqsb {

__device__ __forceinline__ double u_next(const DevSys& s, const double* u0, const double* v0, const double* a0,
                                         int64_t q)
{
    return FQ_ADD(FQ_ADD(u0[q], FQ_MUL(s.dt, v0[q])), FQ_MUL(s.hdt2, a0[q]));
}

/* velocity / acceleration updates of timeStep after the positions, detail.h:1552-1565 */
template <bool UNITS>
__device__ __forceinline__ void verlet_velocity(const DevSys& s, double sfi, double v0, double a0, double& v, double& a,
                                                double& f)
{
    v = FQ_ADD(v0, FQ_MUL(s.dt, a0));
    f = FQ_ADD(sfi, FQ_MUL(s.me, v));
    a = UNITS ? f : FQ_MUL(f, s.inv_m);
#pragma unroll
    for (int rep = 0; rep < 2; ++rep) {
        v = FQ_ADD(v0, FQ_MUL(s.hdt, FQ_ADD(a0, a)));
        f = FQ_ADD(sfi, FQ_MUL(s.me, v));
        a = UNITS ? f : FQ_MUL(f, s.inv_m);
    }
}

__device__ __forceinline__ long long absll(long long x)
{
    return x < 0 ? -x : x;
}

/* Stop tests of one finished step; thread 0 of the last CTA.  sf / sff: sum f^2 and f_frame^2. */
__device__ void finalize_step(const DevSys& s, double uf, double sf, double sff)
{
    Ctl* c = s.ctl;
    int flags = c->flags;
    c->ticket = 0;
    c->step += 1;
    c->inc += 1;
    c->cur ^= 1;
    if (flags & RF_FLOW) {
        c->u_frame = uf;
    }
    if (c->nan_flag) {
        c->error = DERR_NAN;
        return;
    }
    if (c->walk_flag) {
        c->error = DERR_WALK;
        return;
    }
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
    if (flags & RF_EVENT) {
        if (c->a_count != 0) {
            c->done = RUN_EVENT;
            return;
        }
    }
    if (flags & RF_RESID) {
        double r_fres = FQ_SQRT(sf);
        double r_fext = FQ_SQRT(sff);
        double r = r_fext != 0.0 ? FQ_DIV(r_fres, r_fext) : r_fres;
        c->last_residual = r;
        int64_t n = c->niter_tol;
        if (n > 0) {
            double* ring = s.ring;
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
            return;
        }
    }
    if (flags & RF_TRUNCATE) {
        if ((c->A_truncate > 0 && c->a_count >= c->A_truncate) ||
            (c->S_truncate > 0 && c->s_sum >= c->S_truncate)) {
            c->done = RUN_TRUNCATED;
            return;
        }
    }
    if (c->step >= c->max_steps) {
        c->done = RUN_MAXITER;
    }
}

/* Whole-CTA canonical tree over partials[0..G) (zero padded to a power of two). */
__device__ double2 tree_partials(const double2* partials, int64_t G, double* sh)
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
        x = serial_tree([&](int64_t i) { return i < G ? __ldcg(partials + i).x : 0.0; }, lo, per);
        y = serial_tree([&](int64_t i) { return i < G ? __ldcg(partials + i).y : 0.0; }, lo, per);
    }
    double sx = cta_tree(x, sh);
    __syncthreads();
    double sy = cta_tree(y, sh);
    return make_double2(sx, sy);
}

struct StepShared {
    int exit_flag;
    int cur;
    int flags;
    int last;
    int nan;
    double uf;
    unsigned long long ds;
    unsigned long long da;
    double red[32];
};

__device__ __forceinline__ bool step_prologue(const DevSys& s, StepShared& sh)
{
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        volatile Ctl* c = s.ctl;
        sh.exit_flag = (c->done != 0) || (c->error != 0);
        sh.cur = c->cur;
        sh.flags = c->flags;
        double uf = c->u_frame;
        if (sh.flags & RF_FLOW) {
            uf = FQ_ADD(uf, c->vdt);
        }
        sh.uf = uf;
        sh.nan = 0;
        sh.ds = 0ull;
        sh.da = 0ull;
        sh.last = 0;
    }
    __syncthreads();
    return sh.exit_flag == 0;
}

/* Per-particle well check + bookkeeping; returns the (possibly refreshed) well cache. */
__device__ __forceinline__ double4_32a well_of(const DevSys& s, int64_t p, double un, bool act, StepShared& sh)
{
    double4_32a w = s.wc[p];
    if (!(w.x <= un && un < w.y)) {
        int64_t gold = s.gidx[p];
        if (dev_align(s, p, un)) {
            w = s.wc[p];
            int64_t gnew = s.gidx[p];
            if (act && gnew != gold) {
                int64_t ref = s.i_n[p];
                long long ds = absll(gnew - ref) - absll(gold - ref);
                long long da = (long long)(gnew != ref) - (long long)(gold != ref);
                atomicAdd(&sh.ds, (unsigned long long)ds);
                atomicAdd(&sh.da, (unsigned long long)da);
            }
        }
    }
    return w;
}

__device__ __forceinline__ void step_epilogue(const DevSys& s, StepShared& sh, bool finalize_here, double rf,
                                              double rff)
{
    bool resid = (sh.flags & RF_RESID) != 0;
    double sf = 0.0, sff = 0.0;
    if (resid && finalize_here) {
        sf = cta_tree(rf, sh.red);
        __syncthreads();
        sff = cta_tree(rff, sh.red);
    }
    __syncthreads();
    int tid = threadIdx.x + threadIdx.y * blockDim.x;
    int64_t bid = blockIdx.x + (int64_t)blockIdx.y * gridDim.x;
    if (tid == 0) {
        Ctl* c = s.ctl;
        if (resid && finalize_here) {
            s.partials[bid] = make_double2(sf, sff);
        }
        if (sh.ds) {
            atomicAdd((unsigned long long*)&c->s_sum, sh.ds);
        }
        if (sh.da) {
            atomicAdd((unsigned long long*)&c->a_count, sh.da);
        }
        if (sh.nan) {
            atomicOr(&c->nan_flag, 1);
        }
        if (finalize_here) {
            __threadfence();
            unsigned int t = atomicAdd(&c->ticket, 1u);
            sh.last = (t == gridDim.x * gridDim.y - 1);
        }
    }
    if (!finalize_here) {
        return;
    }
    __syncthreads();
    if (sh.last) {
        __threadfence();
        double2 tot = make_double2(0.0, 0.0);
        if (resid) {
            tot = tree_partials(s.partials, (int64_t)gridDim.x * gridDim.y, sh.red);
        }
        if (tid == 0) {
            finalize_step(s, sh.uf, tot.x, tot.y);
        }
    }
}

/*
 * Line1d (INTER_LAPLACE1D) or Particles (INTER_NONE) step.  Thread t of CTA b owns particles
 * b*T*PPT + t*PPT + [0, PPT): a CTA covers an aligned power-of-two range of the flat index, so the
 * residual sums follow the fixed pairwise tree over the flat index.
 */
template <int POT, int INTER, bool UNITS, int PPT>
__global__ void __launch_bounds__(256) k_step_line(DevSys s)
{
    __shared__ StepShared sh;
    __shared__ double sh_un[256 * PPT];
    if (!step_prologue(s, sh)) {
        return;
    }
    const int cur = sh.cur;
    const bool act = (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (sh.flags & RF_RESID) != 0;
    const double uf = sh.uf;
    const int64_t N = s.N;
    const int T = blockDim.x;
    const int64_t base = (int64_t)blockIdx.x * T * PPT;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    double* u1 = s.u[cur ^ 1];
    double* v1 = s.v[cur ^ 1];
    double* a1 = s.a[cur ^ 1];

    double un[PPT], vr[PPT], ar[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        int64_t p = base + threadIdx.x * PPT + j;
        if (p < N) {
            vr[j] = v0[p];
            ar[j] = a0[p];
            un[j] = FQ_ADD(FQ_ADD(u0[p], FQ_MUL(s.dt, vr[j])), FQ_MUL(s.hdt2, ar[j]));
            if (INTER == INTER_LAPLACE1D) {
                sh_un[threadIdx.x * PPT + j] = un[j];
            }
        }
    }
    if (INTER == INTER_LAPLACE1D) {
        __syncthreads();
    }
    double rf = 0.0, rff = 0.0;
    bool nan = false;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        int64_t p = base + threadIdx.x * PPT + j;
        if (p >= N) {
            continue;
        }
        double up = un[j];
        double4_32a w = well_of(s, p, up, act, sh);
        double fp = pot_force<POT, UNITS>(s, w, up);
        double fi = 0.0;
        if (INTER == INTER_LAPLACE1D) {
            int li = threadIdx.x * PPT + j;
            double uL, uR;
            if (li > 0) {
                uL = sh_un[li - 1];
            }
            else {
                uL = u_next(s, u0, v0, a0, p == 0 ? N - 1 : p - 1);
            }
            if (li + 1 < T * PPT && p + 1 < N) {
                uR = sh_un[li + 1];
            }
            else {
                uR = u_next(s, u0, v0, a0, p == N - 1 ? 0 : p + 1);
            }
            fi = FQ_ADD(FQ_SUB(uL, FQ_MUL(2.0, up)), uR);
            if (!UNITS) {
                fi = FQ_MUL(fi, s.k);
            }
        }
        double ff = FQ_MUL(s.k_frame, FQ_SUB(uf, up));
        double sfi = FQ_ADD(FQ_ADD(ff, fp), fi);
        double vv, aa, f;
        verlet_velocity<UNITS>(s, sfi, vr[j], ar[j], vv, aa, f);
        u1[p] = up;
        v1[p] = vv;
        a1[p] = aa;
        nan |= (up != up);
        if (resid) {
            double f2 = FQ_MUL(f, f), ff2 = FQ_MUL(ff, ff);
            if (PPT == 1 || j == 0) {
                rf = f2;
                rff = ff2;
            }
            else {
                rf = FQ_ADD(rf, f2);
                rff = FQ_ADD(rff, ff2);
            }
        }
    }
    if (nan) {
        sh.nan = 1;
    }
    step_epilogue(s, sh, true, rf, rff);
}

/*
 * Line2d step: CTA tile of 8 rows x 32 columns, one particle per thread.  The residual terms are
 * written per particle (sq2) and summed in the flat-index pairwise order by k_reduce_grid, which
 * also finalises the step.
 */
template <int POT, bool UNITS>
__global__ void __launch_bounds__(256) k_step_grid(DevSys s)
{
    __shared__ StepShared sh;
    __shared__ double sh_un[8][32];
    if (!step_prologue(s, sh)) {
        return;
    }
    const int cur = sh.cur;
    const bool act = (sh.flags & (RF_ACT | RF_TRUNCATE | RF_EVENT)) != 0;
    const bool resid = (sh.flags & RF_RESID) != 0;
    const double uf = sh.uf;
    const int64_t R = s.rows, C = s.cols;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t i = (int64_t)blockIdx.y * 8 + ty;
    const int64_t jc = (int64_t)blockIdx.x * 32 + tx;
    const bool valid = i < R && jc < C;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    const int64_t p = i * C + jc;
    double up = 0.0, vr = 0.0, ar = 0.0;
    if (valid) {
        vr = v0[p];
        ar = a0[p];
        up = FQ_ADD(FQ_ADD(u0[p], FQ_MUL(s.dt, vr)), FQ_MUL(s.hdt2, ar));
        sh_un[ty][tx] = up;
    }
    __syncthreads();
    if (valid) {
        double4_32a w = well_of(s, p, up, act, sh);
        double fp = pot_force<POT, UNITS>(s, w, up);
        double uU = ty > 0 ? sh_un[ty - 1][tx] : u_next(s, u0, v0, a0, ((i + R - 1) % R) * C + jc);
        double uD = (ty < 7 && i + 1 < R) ? sh_un[ty + 1][tx] : u_next(s, u0, v0, a0, ((i + 1) % R) * C + jc);
        double uL = tx > 0 ? sh_un[ty][tx - 1] : u_next(s, u0, v0, a0, i * C + (jc + C - 1) % C);
        double uR = (tx < 31 && jc + 1 < C) ? sh_un[ty][tx + 1] : u_next(s, u0, v0, a0, i * C + (jc + 1) % C);
        double fi = FQ_SUB(FQ_ADD(FQ_ADD(FQ_ADD(uU, uD), uL), uR), FQ_MUL(4.0, up));
        if (!UNITS) {
            fi = FQ_MUL(fi, s.k);
        }
        double ff = FQ_MUL(s.k_frame, FQ_SUB(uf, up));
        double sfi = FQ_ADD(FQ_ADD(ff, fp), fi);
        double vv, aa, f;
        verlet_velocity<UNITS>(s, sfi, vr, ar, vv, aa, f);
        s.u[cur ^ 1][p] = up;
        s.v[cur ^ 1][p] = vv;
        s.a[cur ^ 1][p] = aa;
        if (up != up) {
            sh.nan = 1;
        }
        if (resid) {
            s.sq2[p] = make_double2(FQ_MUL(f, f), FQ_MUL(ff, ff));
        }
    }
    step_epilogue(s, sh, false, 0.0, 0.0);
}

/* Pairwise reduction of the 2d step's sq2 in flat-index order (1024 per CTA) + step finalisation. */
__global__ void __launch_bounds__(256) k_reduce_grid(DevSys s)
{
    __shared__ StepShared sh;
    if (!step_prologue(s, sh)) {
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
    step_epilogue(s, sh, true, rf, rff);
}

/* ------------------------------------------------------------- launchers */

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

template <int POT, int INTER>
static cudaError_t launch_line_t(const DevSys& s, const LineGeom& g, bool units, cudaStream_t st)
{
    dim3 grid((unsigned)g.grid), block((unsigned)g.threads);
    if (g.ppt == 2) {
        if (units) {
            k_step_line<POT, INTER, true, 2><<<grid, block, 0, st>>>(s);
        }
        else {
            k_step_line<POT, INTER, false, 2><<<grid, block, 0, st>>>(s);
        }
    }
    else {
        if (units) {
            k_step_line<POT, INTER, true, 1><<<grid, block, 0, st>>>(s);
        }
        else {
            k_step_line<POT, INTER, false, 1><<<grid, block, 0, st>>>(s);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_step_line(const DevSys& s, const LineGeom& g, bool units, cudaStream_t st)
{
    if (s.inter == INTER_LAPLACE1D) {
        switch (s.pot) {
            case POT_CUSPY: return launch_line_t<POT_CUSPY, INTER_LAPLACE1D>(s, g, units, st);
            case POT_SEMISMOOTH: return launch_line_t<POT_SEMISMOOTH, INTER_LAPLACE1D>(s, g, units, st);
            default: return launch_line_t<POT_SMOOTH, INTER_LAPLACE1D>(s, g, units, st);
        }
    }
    switch (s.pot) {
        case POT_CUSPY: return launch_line_t<POT_CUSPY, INTER_NONE>(s, g, units, st);
        case POT_SEMISMOOTH: return launch_line_t<POT_SEMISMOOTH, INTER_NONE>(s, g, units, st);
        default: return launch_line_t<POT_SMOOTH, INTER_NONE>(s, g, units, st);
    }
}

cudaError_t launch_step_grid(const DevSys& s, bool units, cudaStream_t st)
{
    dim3 block(32, 8);
    dim3 grid((unsigned)((s.cols + 31) / 32), (unsigned)((s.rows + 7) / 8));
    switch (s.pot) {
        case POT_CUSPY:
            if (units) {
                k_step_grid<POT_CUSPY, true><<<grid, block, 0, st>>>(s);
            }
            else {
                k_step_grid<POT_CUSPY, false><<<grid, block, 0, st>>>(s);
            }
            break;
        case POT_SEMISMOOTH:
            if (units) {
                k_step_grid<POT_SEMISMOOTH, true><<<grid, block, 0, st>>>(s);
            }
            else {
                k_step_grid<POT_SEMISMOOTH, false><<<grid, block, 0, st>>>(s);
            }
            break;
        default:
            if (units) {
                k_step_grid<POT_SMOOTH, true><<<grid, block, 0, st>>>(s);
            }
            else {
                k_step_grid<POT_SMOOTH, false><<<grid, block, 0, st>>>(s);
            }
            break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        return e;
    }
    k_reduce_grid<<<(unsigned)grid_reduce_ctas(s.N), 256, 0, st>>>(s);
    return cudaGetLastError();
}

} // namespace fqsb
