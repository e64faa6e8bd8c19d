/*
 * Adjoint (reverse mode) of the fused velocity-Verlet step, for gradients of a trajectory loss with
 * respect to the initial positions and velocities, the frame-position schedule, mu, k_interactions
 * and eta.  No counterpart in the reference (which has no derivatives); the forward it differentiates
 * is exactly the reference's timeStep (include/FrictionQPotSpringBlock/detail.h:1539-1570) with
 * u_frame set before every step:
 *
 *   u'  = (u + dt v) + (dt^2/2) a
 *   s   = (f_frame + f_pot) + f_int,  f_frame = k_frame (u_frame - u'),  f_int = k lap(u'),
 *         f_pot = F(u') (Cuspy: mu (c - u') with the forward's well; SemiSmooth: its three branches;
 *         Smooth: -(mu dy / pi) sin(pi (u' - c) / dy))
 *   v1  = v + dt a,            a1 = (s - eta v1) / m
 *   v2  = v + dt/2 (a + a1),   a2 = (s - eta v2) / m
 *   v3  = v + dt/2 (a + a2),   a3 = (s - eta v3) / m         -> (u', v3, a3)
 *
 * One launch processes one step backwards for all particles: phase A recomputes the step's
 * intermediates from the recorded input state, output positions and wells, and pulls the output
 * adjoints (lu, lv, la) back to the force sum (sbar); phase B adds the interaction term
 * k lap(sbar) (the Laplacian is symmetric) and writes the input adjoints.  Per-step gradient terms
 * for u_frame[t], eta, mu and k are summed in the same fixed pairwise order as every other sum here
 * and written to step_out[4 t + {0, 1, 2, 3}].  Cuspy gradients hold the wells fixed at the forward's
 * (the potential is discontinuous at the yield positions); Smooth and SemiSmooth are exact.
 */
#include "fqsb_internal.h"

namespace fqsb {

struct AdjTerms {
    double sbar;   /* dL/ds */
    double upbar;  /* dL/du' without the interaction term */
    double vbar;   /* dL/dv (input) without the position term */
    double abar;   /* dL/da (input) without the position term */
    double gsched; /* k_frame * dL/df_frame */
    double geta, gmu, gk;
};

template <int POT, int INTER>
__device__ __forceinline__ AdjTerms adj_particle(const DevSys& s, const AdjArgs& A, int64_t p)
{
    const int64_t N = s.N;
    AdjTerms r;
    double u = A.u_in[p], v = A.v_in[p], a = A.a_in[p];
    (void)u;
    double up = A.up[p];
    double4_32a w = A.w[p];
    /* forward intermediates.  Smooth: sin and cos of the phase from one sincos call; the adjoint needs
     * them to the gradient tolerance only (the forward's bit-exact sine is not needed here) */
    double fp, sn = 0.0, cs = 0.0;
    if (POT == POT_SMOOTH) {
        const double pi = 3.14159265358979323846;
        double arg = FQ_DIV(FQ_MUL(pi, FQ_SUB(up, w.z)), w.w);
        sincos(arg, &sn, &cs);
        fp = FQ_MUL(FQ_DIV(FQ_MUL(-s.mu, w.w), pi), sn);
    }
    else {
        fp = pot_force<POT>(s, w, up);
    }
    double ff = scale(FQ_SUB(A.uf, up), s.s_kf);
    double lap = 0.0, fi = 0.0;
    if (INTER == INTER_LAPLACE1D) {
        double uL = A.up[p == 0 ? N - 1 : p - 1], uR = A.up[p == N - 1 ? 0 : p + 1];
        lap = FQ_ADD(FQ_SUB(uL, scale_pow2(up, 1, 2.0)), uR);
        fi = scale(lap, s.s_k);
    }
    double sfi = FQ_ADD(FQ_ADD(ff, fp), fi);
    double v1 = FQ_ADD(v, FQ_MUL(s.dt, a));
    double a1 = scale(FQ_ADD(sfi, FQ_MUL(s.me, v1)), s.s_im);
    double v2 = FQ_ADD(v, FQ_MUL(s.hdt, FQ_ADD(a, a1)));
    double a2 = scale(FQ_ADD(sfi, FQ_MUL(s.me, v2)), s.s_im);
    double v3 = FQ_ADD(v, FQ_MUL(s.hdt, FQ_ADD(a, a2)));
    /* reverse */
    const double im = s.inv_m, mim = FQ_MUL(s.me, s.inv_m);
    double la3 = A.la_out[p], lv3 = A.lv_out[p];
    double sb = FQ_MUL(im, la3);
    double geta = -FQ_MUL(FQ_MUL(v3, im), la3);
    lv3 = FQ_ADD(lv3, FQ_MUL(mim, la3));
    double vb = lv3;
    double ab = FQ_MUL(s.hdt, lv3);
    double a2b = FQ_MUL(s.hdt, lv3);
    sb = FQ_ADD(sb, FQ_MUL(im, a2b));
    geta = FQ_SUB(geta, FQ_MUL(FQ_MUL(v2, im), a2b));
    double v2b = FQ_MUL(mim, a2b);
    vb = FQ_ADD(vb, v2b);
    ab = FQ_ADD(ab, FQ_MUL(s.hdt, v2b));
    double a1b = FQ_MUL(s.hdt, v2b);
    sb = FQ_ADD(sb, FQ_MUL(im, a1b));
    geta = FQ_SUB(geta, FQ_MUL(FQ_MUL(v1, im), a1b));
    double v1b = FQ_MUL(mim, a1b);
    vb = FQ_ADD(vb, v1b);
    ab = FQ_ADD(ab, FQ_MUL(s.dt, v1b));
    double ffb = FQ_ADD(sb, A.wff);
    /* dF/du' and dF/dmu */
    double dfdu, dfdmu;
    if (POT == POT_CUSPY) {
        dfdu = -s.mu;
        dfdmu = FQ_SUB(w.z, up);
    }
    else if (POT == POT_SEMISMOOTH) {
        if (up < w.z || up > w.w) {
            dfdu = s.kappa;
            dfdmu = 0.0;
        }
        else {
            dfdu = -s.mu;
            dfdmu = FQ_SUB(FQ_MUL(0.5, FQ_ADD(w.x, w.y)), up);
        }
    }
    else {
        const double pi = 3.14159265358979323846;
        dfdu = -FQ_MUL(s.mu, cs);
        dfdmu = FQ_MUL(FQ_DIV(-w.w, pi), sn);
    }
    r.sbar = sb;
    r.upbar = FQ_ADD(FQ_SUB(A.lu_out[p], scale(ffb, s.s_kf)), FQ_MUL(dfdu, sb));
    r.vbar = vb;
    r.abar = ab;
    r.gsched = scale(ffb, s.s_kf);
    r.geta = geta;
    r.gmu = FQ_MUL(dfdmu, sb);
    r.gk = FQ_MUL(lap, sb);
    return r;
}

template <int POT, int INTER>
__global__ void __launch_bounds__(256) k_adjoint_step(DevSys s, AdjArgs A)
{
    __shared__ double sh_sb[256];
    __shared__ double red[32];
    __shared__ int last;
    const int64_t N = s.N;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    AdjTerms r;
    r.sbar = r.upbar = r.vbar = r.abar = r.gsched = r.geta = r.gmu = r.gk = 0.0;
    if (p < N) {
        r = adj_particle<POT, INTER>(s, A, p);
    }
    sh_sb[threadIdx.x] = r.sbar;
    __syncthreads();
    if (p < N) {
        double upb = r.upbar;
        if (INTER == INTER_LAPLACE1D) {
            int li = threadIdx.x;
            double sL = li > 0 ? sh_sb[li - 1] : adj_particle<POT, INTER>(s, A, p == 0 ? N - 1 : p - 1).sbar;
            double sR = (li + 1 < (int)blockDim.x && p + 1 < N) ? sh_sb[li + 1]
                                                                 : adj_particle<POT, INTER>(s, A, p + 1 == N ? 0 : p + 1).sbar;
            upb = FQ_ADD(upb, scale(FQ_ADD(FQ_SUB(sL, scale_pow2(r.sbar, 1, 2.0)), sR), s.s_k));
        }
        A.lu_in[p] = upb;
        A.lv_in[p] = FQ_ADD(r.vbar, FQ_MUL(s.dt, upb));
        A.la_in[p] = FQ_ADD(r.abar, FQ_MUL(s.hdt2, upb));
    }
    /* per-step gradient terms: pairwise tree over the CTA, then over CTAs by the last CTA */
    double t0 = cta_tree(r.gsched, red);
    __syncthreads();
    double t1 = cta_tree(r.geta, red);
    __syncthreads();
    double t2 = cta_tree(r.gmu, red);
    __syncthreads();
    double t3 = cta_tree(r.gk, red);
    if (threadIdx.x == 0) {
        A.partials[blockIdx.x] = make_double4_32a(t0, t1, t2, t3);
        __threadfence();
        unsigned k = atomicAdd(A.ticket, 1u);
        last = k == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) {
        return;
    }
    __threadfence();
    const int64_t G = gridDim.x;
    const int64_t P = next_pow2(G);
    const int T = blockDim.x;
    double q[4];
    for (int c = 0; c < 4; ++c) {
        double x = 0.0;
        if (P <= T) {
            if ((int64_t)threadIdx.x < G) {
                x = __ldcg(reinterpret_cast<const double*>(A.partials + threadIdx.x) + c);
            }
        }
        else {
            int64_t per = P / T, lo = (int64_t)threadIdx.x * per;
            x = serial_tree(
                [&](int64_t i) {
                    if (i >= G) {
                        return 0.0;
                    }
                    return __ldcg(reinterpret_cast<const double*>(A.partials + i) + c);
                },
                lo, per);
        }
        q[c] = cta_tree(x, red);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        A.step_out[0] = q[0];
        A.step_out[1] = q[1];
        A.step_out[2] = q[2];
        A.step_out[3] = q[3];
        *A.ticket = 0;
    }
}

template <int POT>
static cudaError_t launch_adj_t(const DevSys& s, const AdjArgs& A, cudaStream_t st)
{
    unsigned grid = (unsigned)((s.N + 255) / 256);
    if (s.inter == INTER_LAPLACE1D) {
        k_adjoint_step<POT, INTER_LAPLACE1D><<<grid, 256, 0, st>>>(s, A);
    }
    else {
        k_adjoint_step<POT, INTER_NONE><<<grid, 256, 0, st>>>(s, A);
    }
    return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const DevSys& s, const AdjArgs& A, cudaStream_t st)
{
    switch (s.pot) {
        case POT_CUSPY: return launch_adj_t<POT_CUSPY>(s, A, st);
        case POT_SEMISMOOTH: return launch_adj_t<POT_SEMISMOOTH>(s, A, st);
        default: return launch_adj_t<POT_SMOOTH>(s, A, st);
    }
}

int64_t adjoint_ctas(int64_t N)
{
    return (N + 255) / 256;
}

} // namespace fqsb
