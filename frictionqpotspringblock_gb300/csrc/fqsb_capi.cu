/*
 * C-ABI implementation (include/fqsb.h): handle lifecycle, host<->device transfer, the
 * graph-captured multi-step driver and the small kernels around the fused step
 * (construction of the disorder, alignment, forces on demand, reductions, event-driven
 * helpers, chunk restore).
 *
 * Forces are not stored per step: f_potential, f_interactions, f_frame, f_damping and f are
 * pure functions of (u, v, u_frame, current well, and f_thermal for RandomForcing systems) after
 * every reference operation that calls updated_u / updated_v, so getters recompute them from the
 * state.  The exceptions are System::trigger (detail.h:1972-1977), which returns before updated_u
 * and leaves the forces stale, and RandomNormalForcing::set_f_thermal (detail.h:972-976), which
 * leaves f as it was; the handle then materialises the force arrays and updates them exactly as
 * the reference does (set_u_frame recomputes f_frame and f, set_v / quench / set_inc recompute
 * f_damping and f) until the next operation that calls updated_u.
 */
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fqsb.h"
#include "fqsb_internal.h"

using namespace fqsb;

#define FQSB_VERSION_STRING "fqsb 0.1.0 sm_103a"

struct fqsb_system {
    fqsb_config cfg;
    DevSys d;
    cudaStream_t stream;
    bool own_stream;
    int device;
    bool is2d;
    LineGeom lg;
    /* host mirrors of the run state */
    int cur;
    int64_t inc, qs_first, qs_last;
    double u_frame;
    /* stale-force store (after trigger) */
    bool stored;
    double* fs[5]; /* f_potential, f_interactions, f_frame, f_damping, f */
    /* scratch */
    double* scratch;         /* N doubles */
    double2* red_partials;   /* reduction partials */
    int64_t red_cap;
    double2* red_out;        /* one double2 */
    unsigned long long* mkey;
    int* mflag;
    Ctl* h_ctl;              /* pinned */
    int64_t ring_cap;
    cudaGraphExec_t graph;
    cudaGraphExec_t graph_plain; /* the run graph of runs without activity, residual or recording */
    cudaGraphExec_t graph_resid; /* the run graph of runs with the residual only (minimise) */
    cudaGraphExec_t graph_np; /* the no-passing minimiser's run graph */
    int graph_k;
    bool use_graph; /* false when FQSB_NO_GRAPH=1: host-driven launches (profiling) */
    SmallGeom sg;   /* one-cluster run kernel of small systems */
    bool small_ok;  /* N fits one cluster, 1d ring or no interactions, not disabled by FQSB_NO_SMALL=1 */
    bool nx_dirty;  /* the next-window buffers may be out of date: refresh before the next small run */
    std::string err;
    /* adjoint tape */
    int64_t adj_T, adj_K, adj_last, adj_nseg;
    std::vector<double> adj_sched_host;
    double* adj_sched;
    double* adj_ckpt;   /* nseg x 3 x N */
    double* adj_ffsum;  /* T */
    double* adj_final;  /* 3 x N: state after the forward */
    double adj_final_uframe;
    int64_t adj_final_inc;
};

static std::string g_create_error;

namespace fqsb {
void set_global_error(const std::string& msg)
{
    g_create_error = msg;
}
} // namespace fqsb

static int set_err(fqsb_system* h, int code, const std::string& msg)
{
    if (h) {
        h->err = msg;
    }
    else {
        g_create_error = msg;
    }
    return code;
}

#define CU(h, expr)                                                                                      \
    do {                                                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            return set_err((h), FQSB_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_));        \
        }                                                                                                \
    } while (0)

static inline unsigned blocks_for(int64_t n, int t)
{
    return (unsigned)((n + t - 1) / t);
}

/* ------------------------------------------------------------------ kernels */

__global__ void k_init_chunk(DevSys d)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.N) {
        return;
    }
    d.anc_kind[p] = 0;
    if (d.nx_end) {
        d.nx_end[p] = INT64_MIN; /* no next-window buffer yet */
    }
    double* y = d.data + p * d.W;
    double acc;
    seq_fill(d, p, 0, d.W, y, &acc);
    d.start[p] = 0;
    d.cidx[p] = 0;
    d.gidx[p] = 0;
    d.acc_end[p] = acc;
    d.wc[p] = make_wc(d, y[0], y[1]);
}

__global__ void k_align(DevSys d, const double* u)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        dev_align(d, p, u[p]);
    }
}

/* advanceUniformly detail.h:2027-2050: u += du, then updated_u (align) */
__global__ void k_advance(DevSys d, double* u, double du)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        double x = FQ_ADD(u[p], du);
        u[p] = x;
        dev_align(d, p, x);
    }
}

/* Potential + interaction force of particle p at positions u (reference order, mu applied). */
__device__ __forceinline__ void pi_force(const DevSys& d, const double* u, int64_t p, double& fp, double& fi)
{
    double up = u[p];
    double4_32a w = d.wc[p];
    switch (d.pot) {
        case POT_CUSPY: fp = pot_force<POT_CUSPY>(d, w, up); break;
        case POT_SEMISMOOTH: fp = pot_force<POT_SEMISMOOTH>(d, w, up); break;
        default: fp = pot_force<POT_SMOOTH>(d, w, up); break;
    }
    fi = inter_force_at(d, u, p);
}

/* computeForce with External (detail.h:1326-1328): the thermal force is the last term of the sum */
__device__ __forceinline__ double with_f_thermal(const DevSys& d, int64_t p, double f)
{
    return d.f_th ? FQ_ADD(f, d.f_th[p]) : f;
}

/* all force components of particle p from the state (u, v, u_frame) */
__device__ __forceinline__ void all_forces(const DevSys& d, const double* u, const double* v, double uf, int64_t p,
                                           double* out5)
{
    double fp, fi;
    pi_force(d, u, p, fp, fi);
    double ff = FQ_MUL(d.k_frame, FQ_SUB(uf, u[p]));
    double fd = FQ_MUL(d.me, v[p]);
    out5[0] = fp;
    out5[1] = fi;
    out5[2] = ff;
    out5[3] = fd;
    out5[4] = with_f_thermal(d, p, FQ_ADD(FQ_ADD(FQ_ADD(ff, fp), fi), fd));
}

__global__ void k_forces(DevSys d, const double* u, const double* v, double uf, double* fpot, double* fint,
                         double* fframe, double* fdamp, double* f)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.N) {
        return;
    }
    double o[5];
    all_forces(d, u, v, uf, p, o);
    fpot[p] = o[0];
    fint[p] = o[1];
    fframe[p] = o[2];
    fdamp[p] = o[3];
    f[p] = o[4];
}

/* stored forces: recompute f_frame from the current u (set_u_frame detail.h:1253-1258), then f */
__global__ void k_store_frame(DevSys d, const double* u, double uf, double* fs0, double* fs1, double* fs2, double* fs3,
                              double* fs4)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        double ff = FQ_MUL(d.k_frame, FQ_SUB(uf, u[p]));
        fs2[p] = ff;
        fs4[p] = with_f_thermal(d, p, FQ_ADD(FQ_ADD(FQ_ADD(ff, fs0[p]), fs1[p]), fs3[p]));
    }
}

/* stored forces: recompute f_damping from v (updated_v detail.h:1391-1395), then f */
__global__ void k_store_damp(DevSys d, const double* v, double* fs0, double* fs1, double* fs2, double* fs3,
                             double* fs4)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        double fd = FQ_MUL(d.me, v[p]);
        fs3[p] = fd;
        fs4[p] = with_f_thermal(d, p, FQ_ADD(FQ_ADD(FQ_ADD(fs2[p], fs0[p]), fs1[p]), fd));
    }
}

enum { RED_RESIDUAL = 0, RED_VSQ = 1, RED_FFRAME = 2, RED_USQ = 3 };

/* level 1 of the canonical pairwise reduction: 1024 consecutive particles per CTA (4 per thread) */
__global__ void __launch_bounds__(256) k_reduce_l1(DevSys d, int what, const double* u, const double* v, double uf,
                                                   const double* fs_f, const double* fs_ff, double2* partials)
{
    __shared__ double sh[32];
    int64_t lo = (int64_t)blockIdx.x * 1024 + threadIdx.x * 4;
    double x[4], y[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int64_t p = lo + j;
        x[j] = 0.0;
        y[j] = 0.0;
        if (p < d.N) {
            if (what == RED_VSQ) {
                x[j] = FQ_MUL(v[p], v[p]);
            }
            else if (what == RED_USQ) {
                x[j] = FQ_MUL(u[p], u[p]);
            }
            else {
                double f, ff;
                if (fs_f) {
                    f = fs_f[p];
                    ff = fs_ff[p];
                }
                else {
                    double o[5];
                    all_forces(d, u, v, uf, p, o);
                    f = o[4];
                    ff = o[2];
                }
                if (what == RED_RESIDUAL) {
                    x[j] = FQ_MUL(f, f);
                    y[j] = FQ_MUL(ff, ff);
                }
                else {
                    x[j] = ff;
                }
            }
        }
    }
    double rx = FQ_ADD(FQ_ADD(x[0], x[1]), FQ_ADD(x[2], x[3]));
    double ry = FQ_ADD(FQ_ADD(y[0], y[1]), FQ_ADD(y[2], y[3]));
    double sx = cta_tree(rx, sh);
    __syncthreads();
    double sy = cta_tree(ry, sh);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = make_double2(sx, sy);
    }
}

__global__ void __launch_bounds__(256) k_reduce_l2(const double2* partials, int64_t G, double2* out)
{
    __shared__ double sh[32];
    int64_t P = next_pow2(G);
    int T = blockDim.x;
    double x = 0.0, y = 0.0;
    if (P <= T) {
        if (threadIdx.x < G) {
            x = partials[threadIdx.x].x;
            y = partials[threadIdx.x].y;
        }
    }
    else {
        int64_t per = P / T, lo = (int64_t)threadIdx.x * per;
        x = serial_tree([&](int64_t i) { return i < G ? partials[i].x : 0.0; }, lo, per);
        y = serial_tree([&](int64_t i) { return i < G ? partials[i].y : 0.0; }, lo, per);
    }
    double sx = cta_tree(x, sh);
    __syncthreads();
    double sy = cta_tree(y, sh);
    if (threadIdx.x == 0) {
        *out = make_double2(sx, sy);
    }
}

/* maxUniformDisplacement: Cuspy detail.h:176-187, SemiSmooth :282-334 (min over particles, exact) */
__global__ void k_min_du(DevSys d, const double* u, int direction, unsigned long long* key, int* outside)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.N) {
        return;
    }
    double up = u[p];
    double4_32a w = d.wc[p];
    double du;
    if (d.pot == POT_CUSPY) {
        du = direction > 0 ? FQ_SUB(w.y, up) : FQ_SUB(up, w.x);
    }
    else {
        if (up < w.z || up > w.w) {
            atomicOr(outside, 1);
            return;
        }
        du = direction > 0 ? FQ_SUB(w.w, up) : FQ_SUB(up, w.z);
    }
    /* du >= 0: the IEEE bit pattern orders like the value */
    atomicMin(key, (unsigned long long)__double_as_longlong(du));
}

/* Cuspy::trigger :193-205 / SemiSmooth :339-350 / Smooth :427-438 (after the align, if any) */
__global__ void k_trigger(DevSys d, double* u, int64_t p, double eps, int direction)
{
    double4_32a w = d.wc[p];
    if (direction > 0) {
        u[p] = FQ_ADD(w.y, FQ_MUL(0.5, eps));
    }
    else {
        u[p] = FQ_SUB(w.x, FQ_MUL(0.5, eps));
    }
}

__global__ void k_zero2(double* a, double* b, int64_t n)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        a[p] = 0.0;
        b[p] = 0.0;
    }
}

__global__ void k_fill(double* x, int64_t n, double value)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        x[p] = value;
    }
}

/* sum |index - i_n| and count(index != i_n) (exact integer reductions) */
__global__ void k_index_diff(DevSys d, const int64_t* i_n, long long* s_sum, long long* a_count)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        int64_t diff = d.gidx[p] - i_n[p];
        if (diff != 0) {
            atomicAdd((unsigned long long*)s_sum, (unsigned long long)(long long)(diff < 0 ? -diff : diff));
            atomicAdd((unsigned long long*)a_count, 1ull);
        }
    }
}

/* prrng chunk.restore(state, value, index): the chunk restarts at `index` with data[0] = value */
__global__ void k_restore(DevSys d, const uint64_t* state, const double* value, const int64_t* index)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d.N) {
        return;
    }
    d.anc_kind[p] = 1;
    if (d.nx_end) {
        d.nx_end[p] = INT64_MIN; /* another sequence: the next-window buffer is void */
    }
    d.anc_k[p] = index[p];
    d.anc_state[p] = state[p];
    d.anc_val[p] = value[p];
    double* y = d.data + p * d.W;
    double acc;
    seq_fill(d, p, index[p], d.W, y, &acc);
    d.start[p] = index[p];
    d.cidx[p] = 0;
    d.gidx[p] = index[p];
    d.acc_end[p] = acc;
    d.wc[p] = make_wc(d, y[0], y[1]);
}

__global__ void k_cidx64(const int32_t* c, int64_t* out, int64_t n)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        out[p] = c[p];
    }
}

__global__ void k_wc_lr(const double4_32a* wc, double* left, double* right, int64_t n)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        double4_32a w = wc[p];
        left[p] = w.x;
        right[p] = w.y;
    }
}

/* ------------------------------------------------------------ host pcg32 */

static uint64_t host_pcg_seed(uint64_t initstate)
{
    uint64_t s = 0ULL * PCG_MULT + 1ULL;
    s += initstate;
    return s * PCG_MULT + 1ULL;
}

static uint64_t host_pcg_advance(uint64_t state, uint64_t delta)
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

/* ------------------------------------------------------------ helpers */

/* How the kernels multiply by a parameter c: skip for 1, exponent add for a positive normal power of
 * two, fp64 multiply otherwise (all three give x * c exactly as IEEE multiplication does). */
static Scale classify_scale(double c)
{
    Scale sc;
    sc.c = c;
    sc.e = 0;
    sc.mode = SCALE_GENERAL;
    if (c == 1.0) {
        sc.mode = SCALE_ONE;
        return sc;
    }
    int e = 0;
    double m = std::frexp(c, &e);
    if (c > 0.0 && m == 0.5 && std::isnormal(c)) {
        sc.mode = SCALE_POW2;
        sc.e = e - 1;
    }
    return sc;
}

/* state arrays are padded so that a CTA's vector loads of a partial last tile stay in bounds */
static int64_t padded(int64_t n)
{
    return (n + 1023) / 1024 * 1024;
}

static double* cur_u(fqsb_system* h)
{
    return h->d.u[h->cur];
}
static double* cur_v(fqsb_system* h)
{
    return h->d.v[h->cur];
}
static double* cur_a(fqsb_system* h)
{
    return h->d.a[h->cur];
}

static int sync(fqsb_system* h)
{
    CU(h, cudaStreamSynchronize(h->stream));
    return FQSB_OK;
}

static int align_all(fqsb_system* h)
{
    k_align<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_u(h));
    CU(h, cudaGetLastError());
    return FQSB_OK;
}

/* updated_u: forces become derived from the state again */
static int updated_u(fqsb_system* h)
{
    h->stored = false;
    return align_all(h);
}

static int ensure_red(fqsb_system* h, int64_t G)
{
    if (h->red_cap < G) {
        if (h->red_partials) {
            cudaFree(h->red_partials);
        }
        h->red_partials = nullptr;
        CU(h, cudaMalloc(&h->red_partials, sizeof(double2) * (size_t)G));
        h->red_cap = G;
    }
    return FQSB_OK;
}

/* canonical pairwise reduction; result in *out (host) */
static int reduce(fqsb_system* h, int what, double2* out)
{
    int64_t G = (h->d.N + 1023) / 1024;
    int rc = ensure_red(h, G);
    if (rc) {
        return rc;
    }
    const double* fs_f = h->stored ? h->fs[4] : nullptr;
    const double* fs_ff = h->stored ? h->fs[2] : nullptr;
    k_reduce_l1<<<(unsigned)G, 256, 0, h->stream>>>(h->d, what, cur_u(h), cur_v(h), h->u_frame, fs_f, fs_ff,
                                                    h->red_partials);
    CU(h, cudaGetLastError());
    k_reduce_l2<<<1, 256, 0, h->stream>>>(h->red_partials, G, h->red_out);
    CU(h, cudaGetLastError());
    CU(h, cudaMemcpyAsync(out, h->red_out, sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

static int materialise_forces(fqsb_system* h)
{
    if (h->stored) {
        return FQSB_OK;
    }
    for (int i = 0; i < 5; ++i) {
        if (!h->fs[i]) {
            CU(h, cudaMalloc(&h->fs[i], sizeof(double) * (size_t)h->d.N));
        }
    }
    k_forces<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_u(h), cur_v(h), h->u_frame, h->fs[0], h->fs[1],
                                                            h->fs[2], h->fs[3], h->fs[4]);
    CU(h, cudaGetLastError());
    h->stored = true;
    return FQSB_OK;
}

/* ------------------------------------------------------------ run driver */

/* Device time after which a run's graph launch yields back to the host (which relaunches it). */
static const uint64_t RUN_BUDGET_NS = 200ull * 1000ull * 1000ull;
static const int64_t RING_MIN = 1024;

static int ensure_graph(fqsb_system* h, int mode = KMODE_GENERAL)
{
    if (!h->use_graph) {
        h->d.in_graph = 0;
        return FQSB_OK;
    }
    if (mode != KMODE_GENERAL) {
        cudaGraphExec_t* g = mode == KMODE_PLAIN ? &h->graph_plain : &h->graph_resid;
        if (!*g) {
            /* built from a copy: its conditional handles are its own kernels' arguments */
            DevSys d = h->d;
            CU(h, build_run_graph(d, h->lg, g, mode));
        }
        return FQSB_OK;
    }
    if (h->graph) {
        return FQSB_OK;
    }
    CU(h, build_run_graph(h->d, h->lg, &h->graph));
    return FQSB_OK;
}

struct RunResult {
    int done;
    int error;
    int64_t steps;
};

/*
 * Run up to max_steps fused steps with the stop tests selected by flags.  The whole run is one
 * launch of the run graph (a device-side loop); the host synchronises once (plus once per
 * RUN_BUDGET_NS of device time for long runs).
 */
struct RunIO {
    const double* sched = nullptr;
    double* rec_u = nullptr;
    double* rec_v = nullptr;
    double* rec_a = nullptr;
    double4_32a* rec_w = nullptr;
    double* rec_ffsum = nullptr;
};

static int run(fqsb_system* h, int64_t max_steps, int flags, double tol, int64_t niter_tol, double vdt,
               int64_t A_truncate, int64_t S_truncate, const int64_t* i_n_host, RunResult* res,
               const RunIO* io = nullptr, const NopassArgs* np = nullptr)
{
    res->done = RUN_MAXITER;
    res->error = 0;
    res->steps = 0;
    if (max_steps <= 0) {
        return FQSB_OK;
    }
    h->stored = false;
    int rc;
    if ((flags & RF_RESID) && niter_tol > h->ring_cap) {
        if (h->d.ring) {
            cudaFree(h->d.ring);
        }
        h->d.ring = nullptr;
        CU(h, cudaMalloc(&h->d.ring, sizeof(double) * (size_t)niter_tol));
        h->ring_cap = niter_tol;
        if (h->graph) {
            /* the ring pointer is a kernel argument of the graph */
            cudaGraphExecDestroy(h->graph);
            h->graph = nullptr;
        }
        if (h->graph_plain) {
            cudaGraphExecDestroy(h->graph_plain);
            h->graph_plain = nullptr;
        }
        if (h->graph_resid) {
            cudaGraphExecDestroy(h->graph_resid);
            h->graph_resid = nullptr;
        }
        if (h->graph_np) {
            cudaGraphExecDestroy(h->graph_np);
            h->graph_np = nullptr;
        }
    }
    bool use_small = np == nullptr && h->small_ok && io == nullptr && !(flags & (RF_SCHEDULE | RF_RECORD | RF_FFSUM)) &&
                     !((flags & RF_RESID) && niter_tol > SMALL_RING_MAX);
    /* runs without activity, frame-force sums or recording take the specialised step kernels */
    int kmode = KMODE_GENERAL;
    if (np == nullptr && plain_runs_apply(h->d) && !(flags & (RF_FFSUM | RF_ACT | RF_TRUNCATE | RF_EVENT | RF_RECORD))) {
        kmode = (flags & RF_RESID) ? KMODE_RESID : KMODE_PLAIN;
    }
    if (np) {
        if (h->use_graph && !h->graph_np) {
            CU(h, build_nopass_graph(h->d, h->lg, *np, &h->graph_np));
        }
        if (!h->use_graph) {
            h->d.in_graph = 0;
        }
    }
    else if (!use_small) {
        rc = ensure_graph(h, kmode);
        if (rc) {
            return rc;
        }
    }
    Ctl* c = h->h_ctl;
    memset(c, 0, sizeof(Ctl));
    c->max_steps = max_steps;
    c->tol = tol;
    c->tol2 = tol * tol;
    c->niter_tol = niter_tol;
    c->flags = flags;
    c->vdt = vdt;
    c->A_truncate = A_truncate;
    c->S_truncate = S_truncate;
    c->cur = h->cur;
    c->inc = h->inc;
    c->u_frame = h->u_frame;
    c->sl_ge_tol = niter_tol;
    c->sl_ge_tol2 = niter_tol;
    c->init = 1;
    c->qs_first = h->qs_first;
    c->qs_last = h->qs_last;
    c->budget_ns = RUN_BUDGET_NS;
    if (io) {
        c->sched = io->sched;
        c->rec_u = io->rec_u;
        c->rec_v = io->rec_v;
        c->rec_a = io->rec_a;
        c->rec_w = io->rec_w;
        c->rec_ffsum = io->rec_ffsum;
    }
    if ((flags & RF_RESID) && niter_tol > 0) {
        k_fill<<<blocks_for(niter_tol, 128), 128, 0, h->stream>>>(h->d.ring, niter_tol, INFINITY);
        CU(h, cudaGetLastError());
    }
    if (flags & (RF_ACT | RF_EVENT | RF_TRUNCATE)) {
        if (i_n_host) {
            CU(h, cudaMemcpyAsync(h->d.i_n, i_n_host, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyHostToDevice,
                                  h->stream));
        }
        else {
            CU(h, cudaMemcpyAsync(h->d.i_n, h->d.gidx, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyDeviceToDevice,
                                  h->stream));
        }
    }
    CU(h, cudaMemcpyAsync(h->d.ctl, c, sizeof(Ctl), cudaMemcpyHostToDevice, h->stream));
    if (i_n_host && (flags & (RF_ACT | RF_EVENT | RF_TRUNCATE))) {
        k_index_diff<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(h->d, h->d.i_n, (long long*)&h->d.ctl->s_sum,
                                                                    (long long*)&h->d.ctl->a_count);
        CU(h, cudaGetLastError());
    }
    bool first_launch = true;
    for (;;) {
        if (np) {
            if (h->use_graph) {
                CU(h, cudaGraphLaunch(h->graph_np, h->stream));
            }
            else {
                DevSys d = h->d;
                d.in_graph = 0;
                for (int i = 0; i < 64; ++i) {
                    CU(h, launch_nopass_iteration(d, h->lg, *np, h->stream));
                }
            }
        }
        else if (use_small) {
            if (h->nx_dirty) {
                CU(h, launch_next_window(h->d, h->stream));
                h->nx_dirty = false;
            }
            cudaError_t le = launch_small_run(h->d, h->sg, h->stream);
            if (first_launch && (le == cudaErrorInvalidClusterSize || le == cudaErrorLaunchOutOfResources)) {
                /* the cluster could not be scheduled now (nothing ran): this handle uses the graph path */
                cudaGetLastError();
                h->small_ok = false;
                use_small = false;
                rc = ensure_graph(h, kmode);
                if (rc) {
                    return rc;
                }
                continue;
            }
            CU(h, le);
        }
        else if (h->use_graph) {
            CU(h, cudaGraphLaunch(kmode == KMODE_PLAIN ? h->graph_plain
                                  : kmode == KMODE_RESID ? h->graph_resid
                                                         : h->graph,
                                  h->stream));
        }
        else {
            for (int i = 0; i < 64; ++i) {
                CU(h, launch_iteration(h->d, h->lg, h->stream, kmode));
            }
        }
        first_launch = false;
        CU(h, cudaMemcpyAsync(c, h->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, h->stream));
        rc = sync(h);
        if (rc) {
            return rc;
        }
        if (use_small && c->nx_stale) {
            h->nx_dirty = true;
        }
        if (c->done || c->error) {
            break;
        }
        /* the launch used up its device-time budget: start a new launch window */
        int64_t zero = 0;
        CU(h, cudaMemcpyAsync(&h->d.ctl->launch_steps, &zero, sizeof(zero), cudaMemcpyHostToDevice, h->stream));
    }
    h->cur = c->cur;
    h->inc = c->inc;
    h->u_frame = c->u_frame;
    if (flags & (RF_ACT | RF_TRUNCATE)) {
        h->qs_first = c->qs_first;
        h->qs_last = c->qs_last;
    }
    res->done = c->done ? c->done : RUN_MAXITER;
    res->error = c->error;
    res->steps = c->step;
    if (c->error == DERR_NAN) {
        return set_err(h, FQSB_ERR_NAN, "NaN entries found");
    }
    if (c->error == DERR_WALK) {
        return set_err(h, FQSB_ERR_TIMEOUT, "yield search exceeded its bound (position too far from the chunk)");
    }
    return FQSB_OK;
}

static int quench_impl(fqsb_system* h)
{
    k_zero2<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(cur_v(h), cur_a(h), h->d.N);
    CU(h, cudaGetLastError());
    if (h->stored) {
        k_store_damp<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_v(h), h->fs[0], h->fs[1], h->fs[2],
                                                                    h->fs[3], h->fs[4]);
        CU(h, cudaGetLastError());
    }
    return FQSB_OK;
}

/* ------------------------------------------------------------ lifecycle */

extern "C" const char* fqsb_version(void)
{
    return FQSB_VERSION_STRING;
}

extern "C" const char* fqsb_last_error(const fqsb_system* h)
{
    return h ? h->err.c_str() : g_create_error.c_str();
}

static void free_all(fqsb_system* h)
{
    if (!h) {
        return;
    }
    DevSys& d = h->d;
    void* ptrs[] = {d.data, d.nx, d.nx_end, d.start, d.cidx, d.gidx, d.wc, d.acc_end, d.anc_kind, d.anc_k, d.anc_state, d.anc_val,
                    d.u[0], d.u[1], d.v[0], d.v[1], d.a[0], d.a[1], d.ctl, d.ring, d.partials, d.i_n, d.sq2,
                    d.cta_pending, d.regen_list, (void*)d.lr_pref, d.f_th, d.th_next, (void*)d.th_dinc, d.th_cnt,
                    d.th_list, d.th,
                    (void*)d.offp, h->scratch, h->red_partials, h->red_out, h->mkey, h->mflag, h->fs[0], h->fs[1],
                    h->fs[2], h->fs[3], h->fs[4], h->adj_sched, h->adj_ckpt, h->adj_ffsum, h->adj_final};
    for (void* p : ptrs) {
        if (p) {
            cudaFree(p);
        }
    }
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
    }
    if (h->graph_plain) {
        cudaGraphExecDestroy(h->graph_plain);
    }
    if (h->graph_resid) {
        cudaGraphExecDestroy(h->graph_resid);
    }
    if (h->graph_np) {
        cudaGraphExecDestroy(h->graph_np);
    }
    if (h->h_ctl) {
        cudaFreeHost(h->h_ctl);
    }
    if (h->own_stream && h->stream) {
        cudaStreamDestroy(h->stream);
    }
    delete h;
}

extern "C" int fqsb_create(const fqsb_config* cfg, fqsb_system** out)
{
    FQSB_API_RANGE();
    if (!cfg || !out) {
        return set_err(nullptr, FQSB_ERR_INVALID, "null argument");
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(nullptr, FQSB_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (cfg->rows < 1 || cfg->cols < 1 || cfg->nchunk < 34 || cfg->n_parameters < 0 || cfg->n_parameters > 4) {
        return set_err(nullptr, FQSB_ERR_INVALID, "invalid shape, nchunk (>= 34) or parameters");
    }
    if (cfg->potential < 0 || cfg->potential > 2 || cfg->interactions < 0 || cfg->interactions > 6) {
        return set_err(nullptr, FQSB_ERR_INVALID, "invalid potential or interactions");
    }
    if (cfg->interactions >= FQSB_QUARTIC1D && cfg->potential != FQSB_CUSPY) {
        return set_err(nullptr, FQSB_ERR_UNSUPPORTED,
                       "the Quartic and LongRange interactions are implemented with the Cuspy potential");
    }
    if ((inter_ring(cfg->interactions) || cfg->interactions == FQSB_LONGRANGE1D) && cfg->rows != 1) {
        return set_err(nullptr, FQSB_ERR_INVALID, "Line1d interactions need rows == 1");
    }
    int dist = cfg->distribution;
    if (!(dist == FQSB_DIST_RANDOM || dist == FQSB_DIST_DELTA || dist == FQSB_DIST_EXPONENTIAL ||
          dist == FQSB_DIST_POWER || dist == FQSB_DIST_PARETO || dist == FQSB_DIST_WEIBULL)) {
        return set_err(nullptr, FQSB_ERR_UNSUPPORTED, "distribution not supported (gamma and normal are not implemented)");
    }
    if (cudaSetDevice(cfg->device) != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, FQSB_ERR_NO_DEVICE, "cudaSetDevice failed");
    }
    fqsb_system* h = new fqsb_system();
    memset(&h->d, 0, sizeof(DevSys));
    for (int i = 0; i < 5; ++i) {
        h->fs[i] = nullptr;
    }
    h->cfg = *cfg;
    h->cfg.offset_per_particle = nullptr;
    h->device = cfg->device;
    h->scratch = nullptr;
    h->red_partials = nullptr;
    h->red_cap = 0;
    h->red_out = nullptr;
    h->mkey = nullptr;
    h->mflag = nullptr;
    h->h_ctl = nullptr;
    h->ring_cap = 0;
    h->graph = nullptr;
    h->graph_plain = nullptr;
    h->graph_resid = nullptr;
    h->graph_np = nullptr;
    h->graph_k = 0;
    {
        const char* ng = getenv("FQSB_NO_GRAPH");
        h->use_graph = !(ng && ng[0] == '1');
    }
    h->adj_T = h->adj_K = h->adj_last = h->adj_nseg = 0;
    h->adj_sched = h->adj_ckpt = h->adj_ffsum = h->adj_final = nullptr;
    h->adj_final_uframe = 0.0;
    h->adj_final_inc = 0;
    h->stored = false;
    h->cur = 0;
    h->inc = 0;
    h->qs_first = 0;
    h->qs_last = 0;
    h->u_frame = 0.0;
    if (cfg->stream) {
        h->stream = (cudaStream_t)cfg->stream;
        h->own_stream = false;
    }
    else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return set_err(nullptr, FQSB_ERR_CUDA, "cudaStreamCreate failed");
        }
        h->own_stream = true;
    }
    DevSys& d = h->d;
    int64_t N = cfg->rows * cfg->cols;
    d.N = N;
    d.rows = cfg->rows;
    d.cols = cfg->cols;
    d.pot = cfg->potential;
    d.inter = cfg->interactions;
    d.dt = cfg->dt;
    d.hdt = 0.5 * cfg->dt;
    d.hdt2 = 0.5 * cfg->dt * cfg->dt;
    d.mu = cfg->mu;
    d.kappa = cfg->kappa;
    d.k = cfg->k_interactions;
    d.ia = cfg->interaction_parameters[0];
    d.ib = cfg->interaction_parameters[1];
    d.k4_4 = 0.25 * d.ib;            /* QuarticGradient1d::m_k4_4, detail.h:633 */
    {
        const double mk4_3 = d.ib / 3.0; /* QuarticGradient2d::force, detail.h:685-686 */
        d.qg_c2 = d.ia + mk4_3;
        d.qg_k23 = 2.0 * mk4_3;
    }
    d.k_frame = cfg->k_frame;
    d.me = -cfg->eta;
    d.m = cfg->m;
    d.inv_m = 1.0 / cfg->m;
    d.W = cfg->nchunk;
    d.n0 = cfg->nchunk;
    d.dist = dist;
    d.npar = cfg->n_parameters;
    for (int i = 0; i < 4; ++i) {
        d.par[i] = i < cfg->n_parameters ? cfg->parameters[i] : 0.0;
    }
    d.offset = cfg->offset;
    d.seed = cfg->seed;
    d.buffer = 2;
    d.margin = 30;
    d.min_margin = 6;
    h->is2d = inter_grid(cfg->interactions);
    d.s_mu = classify_scale(d.mu);
    d.s_k = classify_scale(d.k);
    d.s_kf = classify_scale(d.k_frame);
    d.s_im = classify_scale(d.inv_m);
    h->lg = line_geometry(N);
    {
        /* small Line1d / Particles systems: whole runs in one thread-block cluster */
        const char* ns = getenv("FQSB_NO_SMALL");
        const char* nc = getenv("FQSB_SMALL_CTAS");
        int max_ctas = nc ? atoi(nc) : SMALL_MAX_CTAS;
        h->sg = small_geometry(N, max_ctas);
        if (h->sg.ok && h->sg.ctas > 8 && !small_cluster_fits(d, h->sg)) {
            h->sg = small_geometry(N, 8); /* the GPU cannot co-schedule a cluster of 16 */
        }
        h->small_ok = h->sg.ok && !inter_grid(cfg->interactions) && cfg->interactions != FQSB_LONGRANGE1D &&
                      !(ns && ns[0] == '1');
    }
    int64_t nsteps_cta = step_ctas(d, h->lg);
    int64_t npart = h->is2d ? std::max(grid_reduce_ctas(N), nsteps_cta) : h->lg.grid;
    npart = std::max(npart, (int64_t)SMALL_MAX_CTAS); /* the one-cluster run kernel's CTA subtrees */
    d.npartials = npart;

#define ALLOC(ptr, bytes)                                                                                \
    do {                                                                                                 \
        cudaError_t e_ = cudaMalloc((void**)&(ptr), (bytes));                                            \
        if (e_ != cudaSuccess) {                                                                         \
            std::string m_ = std::string("device allocation failed: ") + cudaGetErrorString(e_);         \
            free_all(h);                                                                                 \
            return set_err(nullptr, FQSB_ERR_CUDA, m_);                                                  \
        }                                                                                                \
    } while (0)

    size_t nd = sizeof(double) * (size_t)N;
    size_t ndp = sizeof(double) * (size_t)padded(N);
    ALLOC(d.data, sizeof(double) * (size_t)N * (size_t)d.W);
    if (h->small_ok && N * d.W <= NX_MAX_VALUES) {
        ALLOC(d.nx, sizeof(double) * (size_t)N * (size_t)d.W);
        ALLOC(d.nx_end, sizeof(int64_t) * (size_t)N);
        h->nx_dirty = true;
    }
    ALLOC(d.start, sizeof(int64_t) * (size_t)N);
    ALLOC(d.cidx, sizeof(int32_t) * (size_t)N);
    ALLOC(d.gidx, sizeof(int64_t) * (size_t)N);
    ALLOC(d.wc, sizeof(double4_32a) * (size_t)N);
    ALLOC(d.acc_end, nd);
    ALLOC(d.anc_kind, (size_t)N);
    ALLOC(d.anc_k, sizeof(int64_t) * (size_t)N);
    ALLOC(d.anc_state, sizeof(uint64_t) * (size_t)N);
    ALLOC(d.anc_val, nd);
    for (int b = 0; b < 2; ++b) {
        ALLOC(d.u[b], ndp);
        ALLOC(d.v[b], ndp);
        ALLOC(d.a[b], ndp);
    }
    ALLOC(d.ctl, sizeof(Ctl));
    ALLOC(d.partials, sizeof(double2) * (size_t)npart);
    if (d.inter == INTER_LONGRANGE1D) {
        /* LongRange1d constructor, detail.h:828-841: k / std::pow(d, alpha + 1) on the host */
        std::vector<double> pref((size_t)N);
        for (int64_t dd = 0; dd < N; ++dd) {
            pref[(size_t)dd] = dd == 0 ? 0.0 : d.k / std::pow((double)dd, d.ia + 1.0);
        }
        double* dp = nullptr;
        ALLOC(dp, sizeof(double) * (size_t)N);
        d.lr_pref = dp;
        d.lr_m = (N - N % 2) / 2;
        if (cudaMemcpy(dp, pref.data(), sizeof(double) * (size_t)N, cudaMemcpyHostToDevice) != cudaSuccess) {
            free_all(h);
            return set_err(nullptr, FQSB_ERR_CUDA, "cudaMemcpy failed");
        }
    }
    ALLOC(d.i_n, sizeof(int64_t) * (size_t)N);
    ALLOC(d.cta_pending, sizeof(int32_t) * (size_t)nsteps_cta);
    ALLOC(d.regen_list, sizeof(int32_t) * (size_t)N);
    ALLOC(d.ring, sizeof(double) * (size_t)RING_MIN);
    h->ring_cap = RING_MIN;
    if (h->is2d) {
        ALLOC(d.sq2, sizeof(double2) * (size_t)N);
    }
    ALLOC(h->scratch, nd);
    ALLOC(h->red_out, sizeof(double2));
    ALLOC(h->mkey, sizeof(unsigned long long));
    ALLOC(h->mflag, sizeof(int));
    if (cfg->offset_per_particle) {
        double* op = nullptr;
        ALLOC(op, nd);
        d.offp = op;
        if (cudaMemcpy(op, cfg->offset_per_particle, nd, cudaMemcpyHostToDevice) != cudaSuccess) {
            free_all(h);
            return set_err(nullptr, FQSB_ERR_CUDA, "copy of offset_per_particle failed");
        }
    }
    if (cudaMallocHost((void**)&h->h_ctl, sizeof(Ctl)) != cudaSuccess) {
        free_all(h);
        return set_err(nullptr, FQSB_ERR_CUDA, "pinned allocation failed");
    }
#undef ALLOC
    /* initSystem detail.h:1096-1139: zeros, disorder, refresh */
    cudaStream_t st = h->stream;
    bool ok = cudaMemsetAsync(d.ctl, 0, sizeof(Ctl), st) == cudaSuccess &&
              cudaMemsetAsync(d.cta_pending, 0, sizeof(int32_t) * (size_t)nsteps_cta, st) == cudaSuccess;
    for (int b = 0; b < 2 && ok; ++b) {
        ok = cudaMemsetAsync(d.u[b], 0, ndp, st) == cudaSuccess && cudaMemsetAsync(d.v[b], 0, ndp, st) == cudaSuccess &&
             cudaMemsetAsync(d.a[b], 0, ndp, st) == cudaSuccess;
    }
    if (!ok) {
        free_all(h);
        return set_err(nullptr, FQSB_ERR_CUDA, "initialisation failed");
    }
    k_init_chunk<<<blocks_for(N, 64), 64, 0, st>>>(d);
    k_align<<<blocks_for(N, 128), 128, 0, st>>>(d, d.u[0]);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        std::string m = std::string("construction failed: ") + cudaGetErrorString(e);
        free_all(h);
        return set_err(nullptr, FQSB_ERR_CUDA, m);
    }
    *out = h;
    return FQSB_OK;
}

extern "C" int fqsb_destroy(fqsb_system* h)
{
    if (h) {
        cudaStreamSynchronize(h->stream);
        free_all(h);
    }
    return FQSB_OK;
}

extern "C" int fqsb_size(const fqsb_system* h, int64_t* n)
{
    if (!h || !n) {
        return FQSB_ERR_INVALID;
    }
    *n = h->d.N;
    return FQSB_OK;
}

extern "C" int fqsb_get_stream(fqsb_system* h, void** stream)
{
    if (!h || !stream) {
        return FQSB_ERR_INVALID;
    }
    *stream = (void*)h->stream;
    return FQSB_OK;
}

/* ------------------------------------------------------------ dynamics */

extern "C" int fqsb_time_steps(fqsb_system* h, uint64_t n)
{
    FQSB_API_RANGE();
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    RunResult r;
    return run(h, (int64_t)n, 0, 0.0, 0, 0.0, 0, 0, nullptr, &r);
}

extern "C" int fqsb_time_step(fqsb_system* h)
{
    return fqsb_time_steps(h, 1);
}

extern "C" int fqsb_flow_steps(fqsb_system* h, uint64_t n, double v_frame)
{
    FQSB_API_RANGE();
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    RunResult r;
    return run(h, (int64_t)n, RF_FLOW, 0.0, 0, v_frame * h->d.dt, 0, 0, nullptr, &r);
}

extern "C" int fqsb_time_steps_until_event(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter,
                                           uint64_t* ret)
{
    FQSB_API_RANGE();
    if (!h || !ret) {
        return FQSB_ERR_INVALID;
    }
    RunResult r;
    int rc = run(h, (int64_t)max_iter, RF_RESID | RF_EVENT, tol, (int64_t)niter_tol, 0.0, 0, 0, nullptr, &r);
    if (rc) {
        return rc;
    }
    if (r.done == RUN_CONVERGED) {
        rc = quench_impl(h);
        if (rc) {
            return rc;
        }
        *ret = 0;
    }
    else if (r.done == RUN_EVENT) {
        *ret = (uint64_t)r.steps;
    }
    else {
        *ret = max_iter + 1;
    }
    return sync(h);
}

static int minimise_common(fqsb_system* h, const int64_t* i_n, uint64_t A, uint64_t S, double tol, uint64_t niter_tol,
                           uint64_t max_iter, int time_activity, int max_iter_is_error, bool truncate, uint64_t* ret)
{
    if (!h || !ret) {
        return FQSB_ERR_INVALID;
    }
    if (!(tol < 1.0)) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed (tol < 1.0)");
    }
    int flags = RF_RESID;
    if (time_activity) {
        flags |= RF_ACT;
    }
    if (truncate) {
        flags |= RF_TRUNCATE | RF_ACT;
    }
    RunResult r;
    int rc = run(h, (int64_t)max_iter, flags, tol, (int64_t)niter_tol, 0.0, (int64_t)A, (int64_t)S, i_n, &r);
    if (rc) {
        return rc;
    }
    if (r.done == RUN_CONVERGED) {
        rc = quench_impl(h);
        if (rc) {
            return rc;
        }
        *ret = 0;
        return sync(h);
    }
    if (r.done == RUN_TRUNCATED) {
        *ret = (uint64_t)r.steps;
        return FQSB_OK;
    }
    *ret = max_iter + 1;
    if (max_iter_is_error) {
        return set_err(h, FQSB_ERR_NO_CONVERGENCE, "No convergence found");
    }
    return FQSB_OK;
}

extern "C" int fqsb_minimise(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                             int max_iter_is_error, uint64_t* ret)
{
    FQSB_API_RANGE();
    return minimise_common(h, nullptr, 0, 0, tol, niter_tol, max_iter, time_activity, max_iter_is_error, false, ret);
}

extern "C" int fqsb_minimise_truncate(fqsb_system* h, const int64_t* i_n, uint64_t A_truncate, uint64_t S_truncate,
                                      double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                                      int max_iter_is_error, uint64_t* ret)
{
    FQSB_API_RANGE();
    if (!i_n) {
        return FQSB_ERR_INVALID;
    }
    if (!time_activity) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed (time_activity)");
    }
    return minimise_common(h, i_n, A_truncate, S_truncate, tol, niter_tol, max_iter, 1, max_iter_is_error, true, ret);
}

__global__ void k_damping_only(DevSys d, const double* v, double* f_damp)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        f_damp[p] = FQ_MUL(d.me, v[p]);
    }
}

/* System_Cuspy_Laplace_Nopassing::minimise, detail.h:1694-1753 (see k_nopass_update). */
extern "C" int fqsb_minimise_nopassing(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter,
                                       int max_iter_is_error, uint64_t* ret)
{
    FQSB_API_RANGE();
    if (!h || !ret) {
        return FQSB_ERR_INVALID;
    }
    if (!(tol < 1.0)) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed (tol < 1.0)");
    }
    if (h->d.pot != POT_CUSPY || h->d.inter != INTER_LAPLACE1D || h->d.N < 2 || h->d.f_th) {
        return set_err(h, FQSB_ERR_INVALID,
                       "the no-passing minimiser needs the athermal Cuspy potential on a Line1d ring, N >= 2");
    }
    for (int i = 0; i < 5; ++i) {
        if (!h->fs[i]) {
            CU(h, cudaMalloc(&h->fs[i], sizeof(double) * (size_t)h->d.N));
        }
    }
    NopassArgs A;
    A.f_pot = h->fs[0];
    A.f_int = h->fs[1];
    A.f_frame = h->fs[2];
    A.f = h->fs[4];
    A.den = 2 * h->d.k + h->d.k_frame + h->d.mu;
    A.ppt = h->lg.ppt;
    RunResult r; /* (the force arrays, kernel arguments of the graph, live as long as the handle) */
    int rc = run(h, (int64_t)max_iter, RF_RESID | RF_NOINC, tol, (int64_t)niter_tol, 0.0, 0, 0, nullptr, &r, nullptr,
                 &A);
    h->qs_first = h->inc;
    h->qs_last = h->inc;
    if (rc) {
        return rc;
    }
    if (r.done == RUN_CONVERGED) {
        h->stored = false; /* after the quench every force is again a function of the state */
        rc = quench_impl(h);
        if (rc) {
            return rc;
        }
        *ret = 0;
        return sync(h);
    }
    /* not converged: the forces are those of the last sweep, f without damping (detail.h:1746) */
    k_damping_only<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(h->d, cur_v(h), h->fs[3]);
    CU(h, cudaGetLastError());
    h->stored = true;
    *ret = max_iter + 1;
    if (max_iter_is_error) {
        int rs = sync(h);
        if (rs) {
            return rs;
        }
        return set_err(h, FQSB_ERR_NO_CONVERGENCE, "No convergence found");
    }
    return sync(h);
}

extern "C" int fqsb_max_uniform_displacement(fqsb_system* h, int direction, double* ret)
{
    if (!h || !ret) {
        return FQSB_ERR_INVALID;
    }
    if (direction != 1 && direction != -1) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed (direction == 1 || direction == -1)");
    }
    if (h->d.pot == POT_SMOOTH) {
        return set_err(h, FQSB_ERR_NOT_POSSIBLE, "Operation not possible.");
    }
    int rc = align_all(h);
    if (rc) {
        return rc;
    }
    unsigned long long init = 0x7ff0000000000000ULL; /* +inf */
    CU(h, cudaMemcpyAsync(h->mkey, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemsetAsync(h->mflag, 0, sizeof(int), h->stream));
    k_min_du<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(h->d, cur_u(h), direction, h->mkey, h->mflag);
    CU(h, cudaGetLastError());
    unsigned long long key = 0;
    int outside = 0;
    CU(h, cudaMemcpyAsync(&key, h->mkey, sizeof(key), cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaMemcpyAsync(&outside, h->mflag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    rc = sync(h);
    if (rc) {
        return rc;
    }
    double du;
    memcpy(&du, &key, sizeof(du));
    *ret = outside ? 0.0 : du;
    return FQSB_OK;
}

/* advanceUniformly detail.h:2027-2050 with input_is_frame = false */
static int advance_uniformly(fqsb_system* h, double du, double* du_frame_out)
{
    double du_particles = du;
    double du_frame = du * (h->d.k_frame + h->d.mu) / h->d.k_frame;
    h->stored = false;
    k_advance<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_u(h), du_particles);
    CU(h, cudaGetLastError());
    h->u_frame += du_frame;
    if (du_frame_out) {
        *du_frame_out = du_frame;
    }
    return FQSB_OK;
}

extern "C" int fqsb_event_driven_step(fqsb_system* h, double eps, int kick, int direction, double* ret)
{
    FQSB_API_RANGE();
    if (!h || !ret) {
        return FQSB_ERR_INVALID;
    }
    if (direction != 1 && direction != -1) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed (direction == 1 || direction == -1)");
    }
    double du = 0.0, out = 0.0;
    int rc;
    if (direction > 0 && !kick) {
        rc = fqsb_max_uniform_displacement(h, direction, &du);
        if (rc) {
            return rc;
        }
        if (du < 0.5 * eps) {
            *ret = 0.0;
            return FQSB_OK;
        }
        rc = advance_uniformly(h, du - 0.5 * eps, &out);
    }
    else if (direction > 0 && kick) {
        rc = advance_uniformly(h, eps, &out);
    }
    else if (!kick) {
        rc = fqsb_max_uniform_displacement(h, direction, &du);
        if (rc) {
            return rc;
        }
        if (du < 0.5 * eps) {
            *ret = 0.0;
            return FQSB_OK;
        }
        rc = advance_uniformly(h, 0.5 * eps - du, &out);
    }
    else {
        rc = advance_uniformly(h, -eps, &out);
    }
    if (rc) {
        return rc;
    }
    *ret = out;
    return sync(h);
}

extern "C" int fqsb_trigger(fqsb_system* h, int64_t p, double eps, int direction)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    if (p < 0 || p >= h->d.N) {
        return set_err(h, FQSB_ERR_INVALID, "assertion failed ((size_type)p < m_N)");
    }
    /* the reference returns before updated_u: keep the forces of the state before the trigger */
    int rc = materialise_forces(h);
    if (rc) {
        return rc;
    }
    if (h->d.pot == POT_CUSPY) {
        rc = align_all(h);
        if (rc) {
            return rc;
        }
    }
    k_trigger<<<1, 1, 0, h->stream>>>(h->d, cur_u(h), p, eps, direction);
    CU(h, cudaGetLastError());
    return sync(h);
}

extern "C" int fqsb_advance_to_fixed_force(fqsb_system* h, double f_frame, int allow_plastic)
{
    FQSB_API_RANGE();
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    CU(h, cudaMemcpyAsync(h->d.i_n, h->d.gidx, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyDeviceToDevice, h->stream));
    double2 s;
    int rc = reduce(h, RED_FFRAME, &s);
    if (rc) {
        return rc;
    }
    double mean = s.x / (double)h->d.N;
    rc = advance_uniformly(h, (f_frame - mean) / h->d.mu, nullptr);
    if (rc) {
        return rc;
    }
    long long* cnt = (long long*)h->scratch;
    CU(h, cudaMemsetAsync(cnt, 0, 2 * sizeof(long long), h->stream));
    k_index_diff<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(h->d, h->d.i_n, cnt, cnt + 1);
    CU(h, cudaGetLastError());
    long long hc[2];
    CU(h, cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, h->stream));
    rc = sync(h);
    if (rc) {
        return rc;
    }
    if (!(allow_plastic || hc[1] == 0)) {
        return set_err(h, FQSB_ERR_REQUIRE,
                       "assertion failed (allow_plastic || xt::all(xt::equal(m_chunk->index_at_align(), i_n)))");
    }
    return FQSB_OK;
}

extern "C" int fqsb_quench(fqsb_system* h)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    int rc = quench_impl(h);
    return rc ? rc : sync(h);
}

/* updated_inc (detail.h:1369-1375): thermal draws at the current inc, then computeForce */
static int updated_inc(fqsb_system* h)
{
    if (!h->d.f_th) {
        return FQSB_OK;
    }
    CU(h, launch_thermal_draw(h->d, 0, h->inc, h->stream));
    if (h->stored) {
        /* f from the stored components (f_damping is -eta v in the store) and the new f_thermal */
        k_store_damp<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_v(h), h->fs[0], h->fs[1], h->fs[2],
                                                                    h->fs[3], h->fs[4]);
        CU(h, cudaGetLastError());
    }
    return FQSB_OK;
}

/* refresh detail.h:1310-1315: updated_u, updated_v, updated_inc */
extern "C" int fqsb_refresh(fqsb_system* h)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    int rc = updated_u(h);
    if (!rc) {
        rc = updated_inc(h);
    }
    return rc ? rc : sync(h);
}

/* ------------------------------------------------------------ thermal forcing */

extern "C" int fqsb_set_random_forcing(fqsb_system* h, double mean, double stddev, uint64_t seed,
                                       const int64_t* dinc_init, const int64_t* dinc)
{
    FQSB_API_RANGE();
    if (!h || !dinc_init || !dinc) {
        return FQSB_ERR_INVALID;
    }
    DevSys& d = h->d;
    if (d.f_th) {
        return set_err(h, FQSB_ERR_INVALID, "the system already has a RandomNormalForcing");
    }
    if (d.pot != POT_CUSPY || !(d.inter == INTER_LAPLACE1D || d.inter == INTER_QUARTIC1D || d.inter == INTER_NONE)) {
        return set_err(h, FQSB_ERR_UNSUPPORTED,
                       "RandomNormalForcing is implemented for the Cuspy potential with Laplace1d, Quartic1d or no "
                       "interactions");
    }
    const int64_t N = d.N;
    const int64_t G = thermal_tiles(N);
    double* f_th = nullptr;
    int64_t *next = nullptr, *di = nullptr, *cnt = nullptr;
    int32_t* list = nullptr;
    Thermal* th = nullptr;
    cudaError_t e = cudaMalloc(&f_th, sizeof(double) * (size_t)padded(N));
    if (e == cudaSuccess) {
        e = cudaMalloc(&next, sizeof(int64_t) * (size_t)N);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&di, sizeof(int64_t) * (size_t)N);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&cnt, sizeof(int64_t) * (size_t)G);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&list, sizeof(int32_t) * (size_t)N);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&th, sizeof(Thermal));
    }
    /* prrng pcg32(seed): the PCG seeding procedure on the default stream */
    Thermal t0;
    t0.inc = (PCG_DEFAULT_STREAM << 1u) | 1u;
    t0.state = 0u;
    t0.state = t0.state * PCG_MULT + t0.inc;
    t0.state += seed;
    t0.state = t0.state * PCG_MULT + t0.inc;
    t0.base = t0.state;
    t0.total = 0;
    t0.ticket = 0u;
    t0.pad = 0u;
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(f_th, 0, sizeof(double) * (size_t)padded(N), h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(next, dinc_init, sizeof(int64_t) * (size_t)N, cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(di, dinc, sizeof(int64_t) * (size_t)N, cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(th, &t0, sizeof(Thermal), cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    if (e != cudaSuccess) {
        for (void* q : {(void*)f_th, (void*)next, (void*)di, (void*)cnt, (void*)list, (void*)th}) {
            if (q) {
                cudaFree(q);
            }
        }
        return set_err(h, FQSB_ERR_CUDA, std::string("RandomNormalForcing allocation failed: ") + cudaGetErrorString(e));
    }
    d.f_th = f_th;
    d.th_next = next;
    d.th_dinc = di;
    d.th_cnt = cnt;
    d.th_list = list;
    d.th = th;
    d.th_mean = mean;
    d.th_sc = stddev * M_SQRT2; /* the association of the reference's normal transform */
    /* the run graph's kernels take the new pointers; the one-cluster kernel has no thermal term */
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (h->graph_plain) {
        cudaGraphExecDestroy(h->graph_plain);
        h->graph_plain = nullptr;
    }
    if (h->graph_resid) {
        cudaGraphExecDestroy(h->graph_resid);
        h->graph_resid = nullptr;
    }
    h->small_ok = false;
    int rc = updated_inc(h); /* the constructor's refresh */
    return rc ? rc : sync(h);
}

extern "C" int fqsb_random_forcing_get(fqsb_system* h, uint64_t* state, double* f_thermal, int64_t* next)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    if (!h->d.f_th) {
        return set_err(h, FQSB_ERR_INVALID, "the system has no RandomNormalForcing");
    }
    if (state) {
        CU(h, cudaMemcpyAsync(state, &h->d.th->state, sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
    }
    if (f_thermal) {
        CU(h, cudaMemcpyAsync(f_thermal, h->d.f_th, sizeof(double) * (size_t)h->d.N, cudaMemcpyDeviceToHost,
                              h->stream));
    }
    if (next) {
        CU(h, cudaMemcpyAsync(next, h->d.th_next, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyDeviceToHost,
                              h->stream));
    }
    return sync(h);
}

extern "C" int fqsb_random_forcing_set(fqsb_system* h, const uint64_t* state, const double* f_thermal,
                                       const int64_t* next)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    if (!h->d.f_th) {
        return set_err(h, FQSB_ERR_INVALID, "the system has no RandomNormalForcing");
    }
    if (state) {
        CU(h, cudaMemcpyAsync(&h->d.th->state, state, sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    }
    if (f_thermal) {
        /* set_f_thermal (detail.h:972-976) does not recompute f: keep the forces of before */
        int rc = materialise_forces(h);
        if (rc) {
            return rc;
        }
        CU(h, cudaMemcpyAsync(h->d.f_th, f_thermal, sizeof(double) * (size_t)h->d.N, cudaMemcpyHostToDevice,
                              h->stream));
    }
    if (next) {
        CU(h, cudaMemcpyAsync(h->d.th_next, next, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyHostToDevice,
                              h->stream));
    }
    return sync(h);
}

/* ------------------------------------------------------------ state */

static double* field_dev(fqsb_system* h, int field, int* rc)
{
    *rc = FQSB_OK;
    switch (field) {
        case FQSB_FIELD_U: return cur_u(h);
        case FQSB_FIELD_V: return cur_v(h);
        case FQSB_FIELD_A: return cur_a(h);
        default: break;
    }
    if (field < FQSB_FIELD_F || field > FQSB_FIELD_F_DAMPING) {
        *rc = set_err(h, FQSB_ERR_INVALID, "unknown field");
        return nullptr;
    }
    static const int map[5] = {4, 0, 1, 2, 3}; /* f, f_potential, f_interactions, f_frame, f_damping */
    int slot = map[field - FQSB_FIELD_F];
    if (h->stored) {
        return h->fs[slot];
    }
    /* derived from the state: compute all five into the store arrays without switching to stored mode */
    for (int i = 0; i < 5; ++i) {
        if (!h->fs[i]) {
            if (cudaMalloc(&h->fs[i], sizeof(double) * (size_t)h->d.N) != cudaSuccess) {
                *rc = set_err(h, FQSB_ERR_CUDA, "allocation failed");
                return nullptr;
            }
        }
    }
    k_forces<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_u(h), cur_v(h), h->u_frame, h->fs[0], h->fs[1],
                                                            h->fs[2], h->fs[3], h->fs[4]);
    if (cudaGetLastError() != cudaSuccess) {
        *rc = set_err(h, FQSB_ERR_CUDA, "force kernel failed");
        return nullptr;
    }
    return h->fs[slot];
}

static int get_field_impl(fqsb_system* h, int field, double* out, cudaMemcpyKind kind)
{
    if (!h || !out) {
        return FQSB_ERR_INVALID;
    }
    int rc;
    double* src = field_dev(h, field, &rc);
    if (rc) {
        return rc;
    }
    CU(h, cudaMemcpyAsync(out, src, sizeof(double) * (size_t)h->d.N, kind, h->stream));
    return sync(h);
}

static int set_field_impl(fqsb_system* h, int field, const double* in, cudaMemcpyKind kind)
{
    if (!h || !in) {
        return FQSB_ERR_INVALID;
    }
    if (field < FQSB_FIELD_U || field > FQSB_FIELD_A) {
        return set_err(h, FQSB_ERR_INVALID, "only u, v and a can be set");
    }
    int rc;
    double* dst = field_dev(h, field, &rc);
    CU(h, cudaMemcpyAsync(dst, in, sizeof(double) * (size_t)h->d.N, kind, h->stream));
    if (field == FQSB_FIELD_U) {
        rc = updated_u(h); /* set_u detail.h:1231-1236 */
    }
    else if (field == FQSB_FIELD_V && h->stored) {
        k_store_damp<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_v(h), h->fs[0], h->fs[1], h->fs[2],
                                                                    h->fs[3], h->fs[4]);
        CU(h, cudaGetLastError());
    }
    if (rc) {
        return rc;
    }
    return sync(h);
}

extern "C" int fqsb_get_field(fqsb_system* h, int field, double* out)
{
    return get_field_impl(h, field, out, cudaMemcpyDeviceToHost);
}

extern "C" int fqsb_set_field(fqsb_system* h, int field, const double* in)
{
    return set_field_impl(h, field, in, cudaMemcpyHostToDevice);
}

extern "C" int fqsb_get_field_device(fqsb_system* h, int field, double* out)
{
    return get_field_impl(h, field, out, cudaMemcpyDeviceToDevice);
}

extern "C" int fqsb_set_field_device(fqsb_system* h, int field, const double* in)
{
    return set_field_impl(h, field, in, cudaMemcpyDeviceToDevice);
}

extern "C" int fqsb_get_scalar(fqsb_system* h, int which, double* out)
{
    if (!h || !out) {
        return FQSB_ERR_INVALID;
    }
    double2 s;
    int rc;
    switch (which) {
        case FQSB_SCALAR_U_FRAME:
            *out = h->u_frame;
            return FQSB_OK;
        case FQSB_SCALAR_T:
            *out = (double)h->inc * h->d.dt;
            return FQSB_OK;
        case FQSB_SCALAR_TEMPERATURE:
            rc = reduce(h, RED_VSQ, &s);
            if (rc) {
                return rc;
            }
            *out = 0.5 * h->d.m * s.x / (double)h->d.N;
            return FQSB_OK;
        case FQSB_SCALAR_RESIDUAL: {
            rc = reduce(h, RED_RESIDUAL, &s);
            if (rc) {
                return rc;
            }
            double r_fres = std::sqrt(s.x), r_fext = std::sqrt(s.y);
            *out = r_fext != 0.0 ? r_fres / r_fext : r_fres;
            return FQSB_OK;
        }
        case FQSB_SCALAR_MEAN_F_FRAME:
            rc = reduce(h, RED_FFRAME, &s);
            if (rc) {
                return rc;
            }
            *out = s.x / (double)h->d.N;
            return FQSB_OK;
        default:
            return set_err(h, FQSB_ERR_INVALID, "unknown scalar");
    }
}

extern "C" int fqsb_set_u_frame(fqsb_system* h, double u_frame)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    h->u_frame = u_frame;
    if (h->stored) {
        k_store_frame<<<blocks_for(h->d.N, 128), 128, 0, h->stream>>>(h->d, cur_u(h), h->u_frame, h->fs[0], h->fs[1],
                                                                     h->fs[2], h->fs[3], h->fs[4]);
        CU(h, cudaGetLastError());
        return sync(h);
    }
    return FQSB_OK;
}

extern "C" int fqsb_get_inc(fqsb_system* h, int64_t* inc)
{
    if (!h || !inc) {
        return FQSB_ERR_INVALID;
    }
    *inc = h->inc;
    return FQSB_OK;
}

extern "C" int fqsb_set_inc(fqsb_system* h, int64_t inc)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    h->inc = inc;
    h->qs_first = inc;
    h->qs_last = inc;
    if (h->d.f_th) {
        int rc = updated_inc(h); /* set_inc detail.h:1241-1247 */
        return rc ? rc : sync(h);
    }
    return FQSB_OK;
}

extern "C" int fqsb_set_t(fqsb_system* h, double t)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    h->inc = (int64_t)std::round(t / h->d.dt);
    return FQSB_OK;
}

extern "C" int fqsb_quasistatic_activity(fqsb_system* h, int64_t* first, int64_t* last)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    if (first) {
        *first = h->qs_first;
    }
    if (last) {
        *last = h->qs_last;
    }
    return FQSB_OK;
}

/* ------------------------------------------------------------ chunk */

extern "C" int fqsb_get_index(fqsb_system* h, int64_t* index_at_align, int64_t* chunk_index_at_align,
                              double* left_of_align, double* right_of_align)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    int64_t N = h->d.N;
    if (index_at_align) {
        CU(h, cudaMemcpyAsync(index_at_align, h->d.gidx, sizeof(int64_t) * (size_t)N, cudaMemcpyDeviceToHost,
                              h->stream));
    }
    if (chunk_index_at_align) {
        int64_t* tmp = (int64_t*)h->scratch;
        k_cidx64<<<blocks_for(N, 256), 256, 0, h->stream>>>(h->d.cidx, tmp, N);
        CU(h, cudaGetLastError());
        CU(h, cudaMemcpyAsync(chunk_index_at_align, tmp, sizeof(int64_t) * (size_t)N, cudaMemcpyDeviceToHost,
                              h->stream));
        int rc = sync(h);
        if (rc) {
            return rc;
        }
    }
    if (left_of_align || right_of_align) {
        double* l = nullptr;
        double* r = nullptr;
        CU(h, cudaMallocAsync((void**)&l, sizeof(double) * (size_t)N, h->stream));
        CU(h, cudaMallocAsync((void**)&r, sizeof(double) * (size_t)N, h->stream));
        k_wc_lr<<<blocks_for(N, 256), 256, 0, h->stream>>>(h->d.wc, l, r, N);
        CU(h, cudaGetLastError());
        if (left_of_align) {
            CU(h, cudaMemcpyAsync(left_of_align, l, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
        }
        if (right_of_align) {
            CU(h, cudaMemcpyAsync(right_of_align, r, sizeof(double) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
        }
        CU(h, cudaFreeAsync(l, h->stream));
        CU(h, cudaFreeAsync(r, h->stream));
    }
    return sync(h);
}

extern "C" int fqsb_chunk_size(fqsb_system* h, int64_t* nchunk)
{
    if (!h || !nchunk) {
        return FQSB_ERR_INVALID;
    }
    *nchunk = h->d.W;
    return FQSB_OK;
}

extern "C" int fqsb_chunk_data(fqsb_system* h, double* data, int64_t* start)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    if (data) {
        CU(h, cudaMemcpyAsync(data, h->d.data, sizeof(double) * (size_t)h->d.N * (size_t)h->d.W,
                              cudaMemcpyDeviceToHost, h->stream));
    }
    if (start) {
        CU(h, cudaMemcpyAsync(start, h->d.start, sizeof(int64_t) * (size_t)h->d.N, cudaMemcpyDeviceToHost, h->stream));
    }
    return sync(h);
}

extern "C" int fqsb_chunk_state_at(fqsb_system* h, const int64_t* index, uint64_t* state)
{
    if (!h || !index || !state) {
        return FQSB_ERR_INVALID;
    }
    int64_t N = h->d.N;
    std::vector<uint8_t> kind((size_t)N);
    std::vector<int64_t> ak((size_t)N);
    std::vector<uint64_t> as((size_t)N);
    CU(h, cudaMemcpyAsync(kind.data(), h->d.anc_kind, (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaMemcpyAsync(ak.data(), h->d.anc_k, sizeof(int64_t) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaMemcpyAsync(as.data(), h->d.anc_state, sizeof(uint64_t) * (size_t)N, cudaMemcpyDeviceToHost, h->stream));
    int rc = sync(h);
    if (rc) {
        return rc;
    }
    for (int64_t p = 0; p < N; ++p) {
        if (kind[(size_t)p]) {
            state[p] = host_pcg_advance(as[(size_t)p], (uint64_t)(index[p] - ak[(size_t)p]));
        }
        else {
            state[p] = host_pcg_advance(host_pcg_seed(h->d.seed + (uint64_t)p), (uint64_t)index[p]);
        }
    }
    return FQSB_OK;
}

extern "C" int fqsb_chunk_restore(fqsb_system* h, const uint64_t* state, const double* value, const int64_t* index)
{
    if (!h || !state || !value || !index) {
        return FQSB_ERR_INVALID;
    }
    int64_t N = h->d.N;
    void* buf = nullptr;
    size_t bytes = (sizeof(uint64_t) + sizeof(double) + sizeof(int64_t)) * (size_t)N;
    CU(h, cudaMallocAsync(&buf, bytes, h->stream));
    uint64_t* ds = (uint64_t*)buf;
    double* dv = (double*)(ds + N);
    int64_t* di = (int64_t*)(dv + N);
    CU(h, cudaMemcpyAsync(ds, state, sizeof(uint64_t) * (size_t)N, cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(dv, value, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(di, index, sizeof(int64_t) * (size_t)N, cudaMemcpyHostToDevice, h->stream));
    k_restore<<<blocks_for(N, 64), 64, 0, h->stream>>>(h->d, ds, dv, di);
    CU(h, cudaGetLastError());
    h->nx_dirty = true;
    CU(h, cudaFreeAsync(buf, h->stream));
    return sync(h);
}

/* ------------------------------------------------------------ parameters */

__global__ void k_rewell(DevSys d)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < d.N) {
        const double* y = d.data + p * d.W + d.cidx[p];
        d.wc[p] = make_wc(d, y[0], y[1]);
    }
}

extern "C" int fqsb_set_parameters(fqsb_system* h, double mu, double k_interactions, double eta)
{
    if (!h) {
        return FQSB_ERR_INVALID;
    }
    h->d.mu = mu;
    h->d.k = k_interactions;
    h->d.me = -eta;
    h->cfg.mu = mu;
    h->cfg.k_interactions = k_interactions;
    h->cfg.eta = eta;
    h->d.s_mu = classify_scale(mu);
    h->d.s_k = classify_scale(k_interactions);
    /* the cached well constants of SemiSmooth depend on mu */
    k_rewell<<<blocks_for(h->d.N, 256), 256, 0, h->stream>>>(h->d);
    CU(h, cudaGetLastError());
    if (h->graph_np) {
        cudaGraphExecDestroy(h->graph_np);
        h->graph_np = nullptr;
    }
    if (h->graph) {
        cudaGraphExecDestroy(h->graph); /* the parameters are kernel arguments of the run graph */
        h->graph = nullptr;
    }
    if (h->graph_plain) {
        cudaGraphExecDestroy(h->graph_plain);
        h->graph_plain = nullptr;
    }
    if (h->graph_resid) {
        cudaGraphExecDestroy(h->graph_resid);
        h->graph_resid = nullptr;
    }
    h->stored = false;
    return sync(h);
}

/* ------------------------------------------------------------ adjoint */

static int copy_state(fqsb_system* h, double* dst3, bool to_buffer)
{
    size_t nb = sizeof(double) * (size_t)h->d.N;
    int64_t N = h->d.N;
    if (to_buffer) {
        CU(h, cudaMemcpyAsync(dst3, cur_u(h), nb, cudaMemcpyDeviceToDevice, h->stream));
        CU(h, cudaMemcpyAsync(dst3 + N, cur_v(h), nb, cudaMemcpyDeviceToDevice, h->stream));
        CU(h, cudaMemcpyAsync(dst3 + 2 * N, cur_a(h), nb, cudaMemcpyDeviceToDevice, h->stream));
    }
    else {
        CU(h, cudaMemcpyAsync(cur_u(h), dst3, nb, cudaMemcpyDeviceToDevice, h->stream));
        CU(h, cudaMemcpyAsync(cur_v(h), dst3 + N, nb, cudaMemcpyDeviceToDevice, h->stream));
        CU(h, cudaMemcpyAsync(cur_a(h), dst3 + 2 * N, nb, cudaMemcpyDeviceToDevice, h->stream));
        int rc = updated_u(h); /* set_u: re-align the wells to the restored positions */
        if (rc) {
            return rc;
        }
    }
    return FQSB_OK;
}

extern "C" int fqsb_adjoint_forward(fqsb_system* h, const double* schedule, int64_t T, int64_t K, int64_t last,
                                    double* loss)
{
    FQSB_API_RANGE();
    if (!h || !schedule || !loss || T < 1 || K < 1 || last < 1 || last > T) {
        return FQSB_ERR_INVALID;
    }
    if (h->is2d || h->d.inter == INTER_QUARTIC1D || h->d.inter == INTER_QUARTICGRAD1D ||
        h->d.inter == INTER_LONGRANGE1D || h->d.f_th) {
        return set_err(h, FQSB_ERR_UNSUPPORTED,
                       "the adjoint is implemented for athermal Line1d (Laplace1d) and Particles systems");
    }
    int64_t N = h->d.N;
    int64_t nseg = (T + K - 1) / K;
    for (double* p : {h->adj_sched, h->adj_ckpt, h->adj_ffsum, h->adj_final}) {
        if (p) {
            cudaFree(p);
        }
    }
    h->adj_sched = h->adj_ckpt = h->adj_ffsum = h->adj_final = nullptr;
    CU(h, cudaMalloc(&h->adj_sched, sizeof(double) * (size_t)T));
    CU(h, cudaMalloc(&h->adj_ckpt, sizeof(double) * 3 * (size_t)N * (size_t)nseg));
    CU(h, cudaMalloc(&h->adj_ffsum, sizeof(double) * (size_t)T));
    CU(h, cudaMalloc(&h->adj_final, sizeof(double) * 3 * (size_t)N));
    h->adj_sched_host.assign(schedule, schedule + T);
    CU(h, cudaMemcpyAsync(h->adj_sched, schedule, sizeof(double) * (size_t)T, cudaMemcpyHostToDevice, h->stream));
    h->adj_T = T;
    h->adj_K = K;
    h->adj_last = last;
    h->adj_nseg = nseg;
    for (int64_t seg = 0; seg < nseg; ++seg) {
        int rc = copy_state(h, h->adj_ckpt + 3 * N * seg, true);
        if (rc) {
            return rc;
        }
        RunIO io;
        io.sched = h->adj_sched + seg * K;
        io.rec_ffsum = h->adj_ffsum + seg * K;
        RunResult r;
        rc = run(h, std::min(K, T - seg * K), RF_SCHEDULE | RF_FFSUM, 0.0, 0, 0.0, 0, 0, nullptr, &r, &io);
        if (rc) {
            return rc;
        }
    }
    int rc = copy_state(h, h->adj_final, true);
    if (rc) {
        return rc;
    }
    h->adj_final_uframe = h->u_frame;
    h->adj_final_inc = h->inc;
    std::vector<double> ffs((size_t)T);
    CU(h, cudaMemcpyAsync(ffs.data(), h->adj_ffsum, sizeof(double) * (size_t)T, cudaMemcpyDeviceToHost, h->stream));
    double2 usq;
    rc = reduce(h, RED_USQ, &usq); /* synchronises */
    if (rc) {
        return rc;
    }
    /* L = (1/last) sum_{t >= T-last} mean_p f_frame_t + 0.5 mean_p u_T^2 */
    double acc = 0.0;
    for (int64_t t = T - last; t < T; ++t) {
        acc += ffs[(size_t)t] / (double)N;
    }
    *loss = acc / (double)last + 0.5 * (usq.x / (double)N);
    return FQSB_OK;
}

__global__ void k_adj_init(const double* uT, int64_t N, double* lu, double* lv, double* la)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < N) {
        lu[p] = FQ_DIV(uT[p], (double)N);
        lv[p] = 0.0;
        la[p] = 0.0;
    }
}

/* The backward of fqsb_adjoint_backward / _device: grad_u0 and grad_v0 are copied out with `out_kind`
 * (device-to-host for host buffers, device-to-device for device buffers). */
static int adjoint_backward(fqsb_system* h, double* grad_u0, double* grad_v0, double* grad_schedule,
                            double* grad_params, cudaMemcpyKind out_kind)
{
    if (!h || !grad_u0 || !grad_v0 || !grad_schedule || !grad_params) {
        return FQSB_ERR_INVALID;
    }
    if (h->adj_T < 1) {
        return set_err(h, FQSB_ERR_INVALID, "fqsb_adjoint_backward needs a preceding fqsb_adjoint_forward");
    }
    const int64_t N = h->d.N, T = h->adj_T, K = h->adj_K, last = h->adj_last, nseg = h->adj_nseg;
    const size_t nb = sizeof(double) * (size_t)N;
    double *rec_u = nullptr, *rec_v = nullptr, *rec_a = nullptr, *lam = nullptr, *step_out = nullptr;
    double4_32a *rec_w = nullptr, *parts = nullptr;
    unsigned* ticket = nullptr;
    int rc = FQSB_OK;
    auto cleanup = [&]() {
        for (void* p : {(void*)rec_u, (void*)rec_v, (void*)rec_a, (void*)lam, (void*)step_out, (void*)rec_w,
                        (void*)parts, (void*)ticket}) {
            if (p) {
                cudaFree(p);
            }
        }
    };
#define ACU(expr)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            cleanup();                                                                                   \
            return set_err(h, FQSB_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_));          \
        }                                                                                                \
    } while (0)
    ACU(cudaMalloc(&rec_u, nb * (size_t)K));
    ACU(cudaMalloc(&rec_v, nb * (size_t)K));
    ACU(cudaMalloc(&rec_a, nb * (size_t)K));
    ACU(cudaMalloc(&rec_w, sizeof(double4_32a) * (size_t)N * (size_t)K));
    ACU(cudaMalloc(&lam, nb * 6));
    ACU(cudaMalloc(&step_out, sizeof(double) * 4 * (size_t)T));
    ACU(cudaMalloc(&parts, sizeof(double4_32a) * (size_t)adjoint_ctas(N)));
    ACU(cudaMalloc(&ticket, sizeof(unsigned)));
    ACU(cudaMemsetAsync(ticket, 0, sizeof(unsigned), h->stream));
    double* lin = lam;          /* lu, lv, la of the current step's outputs */
    double* lout = lam + 3 * N; /* written by the step */
    k_adj_init<<<blocks_for(N, 256), 256, 0, h->stream>>>(h->adj_final, N, lin, lin + N, lin + 2 * N);
    ACU(cudaGetLastError());
    const double wff = 1.0 / ((double)last * (double)N);
    for (int64_t seg = nseg - 1; seg >= 0 && rc == FQSB_OK; --seg) {
        const double* ck = h->adj_ckpt + 3 * N * seg;
        rc = copy_state(h, const_cast<double*>(ck), false);
        if (rc) {
            break;
        }
        int64_t Ks = std::min(K, T - seg * K);
        RunIO io;
        io.sched = h->adj_sched + seg * K;
        io.rec_u = rec_u;
        io.rec_v = rec_v;
        io.rec_a = rec_a;
        io.rec_w = rec_w;
        RunResult r;
        rc = run(h, Ks, RF_SCHEDULE | RF_RECORD, 0.0, 0, 0.0, 0, 0, nullptr, &r, &io);
        if (rc) {
            break;
        }
        for (int64_t t = Ks - 1; t >= 0; --t) {
            int64_t gt = seg * K + t;
            AdjArgs A;
            if (t == 0) {
                A.u_in = ck;
                A.v_in = ck + N;
                A.a_in = ck + 2 * N;
            }
            else {
                A.u_in = rec_u + (size_t)(t - 1) * N;
                A.v_in = rec_v + (size_t)(t - 1) * N;
                A.a_in = rec_a + (size_t)(t - 1) * N;
            }
            A.up = rec_u + (size_t)t * N;
            A.w = rec_w + (size_t)t * N;
            A.uf = h->adj_sched_host[(size_t)gt];
            A.wff = gt >= T - last ? wff : 0.0;
            A.lu_out = lin;
            A.lv_out = lin + N;
            A.la_out = lin + 2 * N;
            A.lu_in = lout;
            A.lv_in = lout + N;
            A.la_in = lout + 2 * N;
            A.partials = parts;
            A.step_out = step_out + 4 * gt;
            A.ticket = ticket;
            ACU(launch_adjoint_step(h->d, A, h->stream));
            std::swap(lin, lout);
        }
    }
    if (rc) {
        cleanup();
        return rc;
    }
    std::vector<double> so((size_t)(4 * T));
    ACU(cudaMemcpyAsync(grad_u0, lin, nb, out_kind, h->stream));
    ACU(cudaMemcpyAsync(grad_v0, lin + N, nb, out_kind, h->stream));
    ACU(cudaMemcpyAsync(so.data(), step_out, sizeof(double) * 4 * (size_t)T, cudaMemcpyDeviceToHost, h->stream));
    ACU(cudaStreamSynchronize(h->stream));
    double gmu = 0.0, gk = 0.0, geta = 0.0;
    for (int64_t t = 0; t < T; ++t) {
        grad_schedule[t] = so[(size_t)(4 * t)];
        geta += so[(size_t)(4 * t + 1)];
        gmu += so[(size_t)(4 * t + 2)];
        gk += so[(size_t)(4 * t + 3)];
    }
    grad_params[0] = gmu;
    grad_params[1] = gk;
    grad_params[2] = geta;
    /* leave the system in the forward's final state */
    rc = copy_state(h, h->adj_final, false);
    h->u_frame = h->adj_final_uframe;
    h->inc = h->adj_final_inc;
    cleanup();
#undef ACU
    return rc ? rc : sync(h);
}

extern "C" int fqsb_adjoint_backward(fqsb_system* h, double* grad_u0, double* grad_v0, double* grad_schedule,
                                     double* grad_params)
{
    FQSB_API_RANGE();
    return adjoint_backward(h, grad_u0, grad_v0, grad_schedule, grad_params, cudaMemcpyDeviceToHost);
}

extern "C" int fqsb_adjoint_backward_device(fqsb_system* h, double* grad_u0_device, double* grad_v0_device,
                                            double* grad_schedule, double* grad_params)
{
    FQSB_API_RANGE();
    return adjoint_backward(h, grad_u0_device, grad_v0_device, grad_schedule, grad_params,
                            cudaMemcpyDeviceToDevice);
}
