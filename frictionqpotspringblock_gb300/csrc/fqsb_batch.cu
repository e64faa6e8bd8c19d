/*
 * Batched form: thousands of independent Line1d System_Cuspy_Laplace realisations of uneven size
 * running the quasistatic protocol of the reference's examples (examples/Line1d_Cuspy_Laplace.py:41-60:
 * eventDrivenStep without kick, eventDrivenStep with kick, minimise) in one graph launch.
 *
 * Layout: all realisations' particles are concatenated, each realisation padded to whole tiles
 * (tile = threads x particles-per-thread, a power of two); one CTA = one tile of one realisation.
 * Each realisation has a control block (Inst) with its protocol phase, buffer parity, frame position,
 * StopList window and counters.  Every iteration of the run graph's WHILE loop advances every
 * unfinished realisation by one phase step:
 *   PH_EVT_MIN    maxUniformDisplacement (detail.h:1901-1905, Cuspy :176-187): exact min over particles
 *   PH_EVT_APPLY  advanceUniformly(du - eps/2) (detail.h:1937-1943, 2027-2050)
 *   PH_KICK_APPLY advanceUniformly(eps) (detail.h:1945-1947)
 *   PH_MIN_STEP   one fused timeStep + the minimise stop test (detail.h:1754-1785)
 *   PH_QUENCH     quench (detail.h:1527-1532)
 *   PH_REPORT     mean f_frame, the avalanche size S and inc of the cycle are recorded
 * The CTA that finishes a realisation's phase step last (per-realisation ticket) advances its state
 * machine; convergence is per realisation.  Chunk windows are small (W yields per particle, the
 * logical chunk size n0 fixes the canonical yield sequence), so memory is O(W) per particle; moving a
 * window uses the same regeneration branch as the plain path.
 *
 * Arithmetic is the plain path's exactly (same device functions, same pairwise tree per
 * realisation), so every realisation's trajectory and well indices equal those of the plain path
 * run on it alone -- bit for bit.
 */
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fqsb.h"
#include "fqsb_internal.h"

namespace fqsb {

enum : int { PH_EVT_MIN = 0, PH_EVT_APPLY = 1, PH_KICK_APPLY = 2, PH_MIN_STEP = 3, PH_QUENCH = 4, PH_REPORT = 5,
             PH_DONE = 6 };
enum : int { BST_OK = 0, BST_NAN = 1, BST_NO_CONVERGENCE = 2, BST_WALK = 5 };
constexpr int BATCH_RING = 64; /* StopList window capacity (niter_tol <= 64) */

struct Inst {
    int64_t off, n, tile0, ntiles;
    double k_frame, u_frame;
    Scale s_kf;
    int32_t phase, cycle, cur, status;
    uint32_t ticket, ticket_redo;
    int32_t n_pending, nan_flag;
    int64_t inc, steps, s_signed;
    unsigned long long min_key;
    double du_p, du_frame;
    int64_t sl_pos, sl_ge_tol, sl_ge_tol2, sl_asc;
    double ring[BATCH_RING];
};

struct BatchRun {
    int32_t ncycles, niter_tol;
    double eps, tol, tol2;
    int64_t max_iter;
    uint32_t ticket, ticket_redo;
    int32_t n_pending_tiles, n_regen, active, walk_flag;
    uint64_t launch_t0, budget_ns;
    int64_t launch_iters, iters;
    int32_t n_active_tiles; /* entries of BatchDev::active_tiles: the tiles of unfinished realisations */
    int32_t rebuild;        /* a realisation finished this iteration: rebuild the list at its end */
};

struct BatchDev {
    DevSys d;
    Inst* inst;
    BatchRun* run;
    const int32_t* tile_inst;
    int32_t* active_tiles; /* tile of CTA k of a pass, k < BatchRun::n_active_tiles */
    int64_t ntiles, ninst;
    int tile, ppt;
    double2* partials;
    int32_t* tile_pending;
    int32_t* regen_list;
    double *out_uframe, *out_fframe;
    int64_t *out_S, *out_inc;
    unsigned long long h_while, h_if;
    int in_graph; /* 0: the host launches each pass (FQSB_NO_GRAPH=1 at creation), no conditionals to set */
};

__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct BShared {
    int skip, phase, cur, last_inst, last_glob, pending, nan, nact, tile;
    double uf, du_p;
    unsigned long long ds;
    unsigned long long mkey;
    double red[32];
};

/* canonical tree over the tile partials of one realisation (tiles are aligned subtrees) */
__device__ double2 inst_tree(const double2* partials, int64_t G, double* sh)
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
        int64_t per = P / T, lo = (int64_t)threadIdx.x * per;
        const double2 t = serial_tree2(
            [&](int64_t i) { return i < G ? __ldcg(partials + i) : make_double2(0.0, 0.0); }, lo, per);
        x = t.x;
        y = t.y;
    }
    double sx = cta_tree(x, sh);
    __syncthreads();
    double sy = cta_tree(y, sh);
    return make_double2(sx, sy);
}

/* per-realisation state machine; thread 0 of the realisation's last CTA; tot = tree of tile partials */
__device__ void inst_finalize(const BatchDev& b, Inst* I, int j, double2 tot)
{
    BatchRun* R = b.run;
    const DevSys& s = b.d;
    I->ticket = 0;
    I->ticket_redo = 0;
    I->n_pending = 0;
    int ph = I->phase;
    bool done = false;
    if (ph == PH_MIN_STEP) {
        I->cur ^= 1;
        I->inc += 1;
        I->steps += 1;
        if (I->nan_flag) {
            I->status = BST_NAN;
            done = true;
        }
        else {
            double r_fres = FQ_SQRT(tot.x), r_fext = FQ_SQRT(tot.y);
            double r = r_fext != 0.0 ? FQ_DIV(r_fres, r_fext) : r_fres;
            int64_t n = R->niter_tol;
            if (n > 0) {
                int64_t pos = I->sl_pos;
                double old = I->ring[pos];
                if (old >= R->tol) {
                    I->sl_ge_tol -= 1;
                }
                if (old >= R->tol2) {
                    I->sl_ge_tol2 -= 1;
                }
                if (n >= 2) {
                    if (I->ring[(pos + 1) % n] > old) {
                        I->sl_asc -= 1;
                    }
                    if (r > I->ring[(pos + n - 1) % n]) {
                        I->sl_asc += 1;
                    }
                }
                I->ring[pos] = r;
                I->sl_pos = (pos + 1) % n;
                if (r >= R->tol) {
                    I->sl_ge_tol += 1;
                }
                if (r >= R->tol2) {
                    I->sl_ge_tol2 += 1;
                }
            }
            if ((I->sl_asc == 0 && I->sl_ge_tol == 0) || I->sl_ge_tol2 == 0) {
                I->phase = PH_QUENCH;
            }
            else if (I->steps >= R->max_iter) {
                I->status = BST_NO_CONVERGENCE;
                done = true;
            }
        }
    }
    else if (ph == PH_EVT_MIN) {
        double du = __longlong_as_double((long long)I->min_key);
        I->min_key = 0x7ff0000000000000ULL;
        double heps = FQ_MUL(0.5, R->eps);
        if (du < heps) {
            /* no advance (detail.h:1938-1940); the kick follows */
            I->du_p = R->eps;
            I->du_frame = FQ_DIV(FQ_MUL(R->eps, FQ_ADD(I->k_frame, s.mu)), I->k_frame);
            I->phase = PH_KICK_APPLY;
        }
        else {
            double dp = FQ_SUB(du, heps);
            I->du_p = dp;
            I->du_frame = FQ_DIV(FQ_MUL(dp, FQ_ADD(I->k_frame, s.mu)), I->k_frame);
            I->phase = PH_EVT_APPLY;
        }
    }
    else if (ph == PH_EVT_APPLY || ph == PH_KICK_APPLY) {
        I->cur ^= 1;
        I->u_frame = FQ_ADD(I->u_frame, I->du_frame);
        if (ph == PH_EVT_APPLY) {
            I->du_p = R->eps;
            I->du_frame = FQ_DIV(FQ_MUL(R->eps, FQ_ADD(I->k_frame, s.mu)), I->k_frame);
            I->phase = PH_KICK_APPLY;
        }
        else {
            I->phase = PH_MIN_STEP;
            I->steps = 0;
            I->sl_pos = 0;
            I->sl_ge_tol = R->niter_tol;
            I->sl_ge_tol2 = R->niter_tol;
            I->sl_asc = 0;
            for (int k = 0; k < R->niter_tol; ++k) {
                I->ring[k] = __longlong_as_double(0x7ff0000000000000LL);
            }
        }
    }
    else if (ph == PH_QUENCH) {
        I->phase = PH_REPORT;
    }
    else if (ph == PH_REPORT) {
        int64_t o = (int64_t)j * R->ncycles + I->cycle;
        b.out_uframe[o] = I->u_frame;
        b.out_fframe[o] = FQ_DIV(tot.x, (double)I->n);
        b.out_S[o] = I->s_signed;
        b.out_inc[o] = I->inc;
        I->s_signed = 0;
        I->cycle += 1;
        if (I->cycle < R->ncycles) {
            I->phase = PH_EVT_MIN;
        }
        else {
            done = true;
        }
    }
    if (done) {
        I->phase = PH_DONE;
        atomicSub(&R->active, 1);
        R->rebuild = 1;
    }
    __threadfence();
}

/*
 * The list of tiles that still have work: the tiles of every unfinished realisation, in realisation
 * order (a realisation's tiles stay consecutive, so its tile tickets and partials are unchanged).
 * Run by all threads of the CTA that ends the iteration; each thread takes a contiguous run of
 * realisations, an exclusive scan over the threads places their tiles.
 */
__device__ void rebuild_active_tiles(const BatchDev& b)
{
    __shared__ int64_t scan[256];
    const int T = blockDim.x;
    const int64_t ninst = b.ninst;
    const int64_t per = (ninst + T - 1) / T;
    const int64_t j0 = (int64_t)threadIdx.x * per, j1 = j0 + per < ninst ? j0 + per : ninst;
    int64_t cnt = 0;
    for (int64_t j = j0; j < j1; ++j) {
        const volatile Inst* I = b.inst + j;
        if (I->phase != PH_DONE) {
            cnt += I->ntiles;
        }
    }
    scan[threadIdx.x] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int k = 0; k < T; ++k) {
            int64_t c = scan[k];
            scan[k] = acc;
            acc += c;
        }
        b.run->n_active_tiles = (int32_t)acc;
        b.run->rebuild = 0;
    }
    __syncthreads();
    int64_t o = scan[threadIdx.x];
    for (int64_t j = j0; j < j1; ++j) {
        const volatile Inst* I = b.inst + j;
        if (I->phase != PH_DONE) {
            for (int64_t q = 0; q < I->ntiles; ++q) {
                b.active_tiles[o++] = (int32_t)(I->tile0 + q);
            }
        }
    }
    __threadfence();
}

/* global end of one loop iteration (thread 0 of the grid's last CTA of this pass) */
__device__ void batch_iteration_end(const BatchDev& b, bool redo)
{
    BatchRun* R = b.run;
    if (!redo && R->n_pending_tiles > 0) {
        R->ticket = 0;
        if (b.in_graph) {
            cudaGraphSetConditional((cudaGraphConditionalHandle)b.h_if, 1u);
        }
        return;
    }
    if (!redo) {
        if (b.in_graph) {
            cudaGraphSetConditional((cudaGraphConditionalHandle)b.h_if, 0u);
        }
    }
    R->ticket = 0;
    R->ticket_redo = 0;
    R->n_pending_tiles = 0;
    R->n_regen = 0;
    uint64_t now = gtimer();
    if (R->launch_iters == 0) {
        R->launch_t0 = now;
    }
    R->launch_iters += 1;
    R->iters += 1;
    bool more = R->active > 0 && R->walk_flag == 0 && (now - R->launch_t0) < R->budget_ns;
    __threadfence();
    if (b.in_graph) {
        cudaGraphSetConditional((cudaGraphConditionalHandle)b.h_while, more ? 1u : 0u);
    }
}

/*
 * One phase step of one tile.  Thread t owns the PPT consecutive particles t*PPT + [0, PPT) of the tile;
 * neighbours on the realisation's ring come from shared memory or are recomputed at the tile edges.
 */
template <int PPT>
__global__ void __launch_bounds__(256, 4) k_batch(BatchDev b, int redo)
{
    __shared__ BShared sh;
    __shared__ double sh_un[256 * PPT];
    if (threadIdx.x == 0) {
        /* CTA k takes the k-th tile of an unfinished realisation; the others have nothing to do.  While
         * no realisation has finished the list is the identity (no second dependent load). */
        sh.nact = ((volatile BatchRun*)b.run)->n_active_tiles;
        sh.tile = sh.nact == (int)b.ntiles ? (int)blockIdx.x
                                            : ((int)blockIdx.x < sh.nact ? b.active_tiles[blockIdx.x] : -1);
    }
    __syncthreads();
    if (sh.tile < 0) {
        return;
    }
    const int64_t t = sh.tile;
    const int j = b.tile_inst[t];
    Inst* I = b.inst + j;
    const DevSys& s = b.d;
    if (threadIdx.x == 0) {
        volatile Inst* vi = I;
        sh.phase = vi->phase;
        sh.cur = vi->cur;
        sh.uf = vi->u_frame;
        sh.du_p = vi->du_p;
        sh.skip = redo ? !b.tile_pending[t] : 0;
        sh.pending = 0;
        sh.nan = 0;
        sh.ds = 0ull;
        sh.mkey = 0x7ff0000000000000ULL;
        sh.last_inst = 0;
        sh.last_glob = 0;
    }
    __syncthreads();
    if (sh.skip) {
        return;
    }
    if (redo && threadIdx.x == 0) {
        b.tile_pending[t] = 0;
    }
    const int phase = sh.phase;
    const int cur = sh.cur;
    const int64_t off = I->off, n = I->n;
    const int64_t lbase = (t - I->tile0) * (int64_t)b.tile; /* local index of the tile's first particle */
    const int64_t l0 = lbase + (int64_t)threadIdx.x * PPT;
    const double* u0 = s.u[cur];
    const double* v0 = s.v[cur];
    const double* a0 = s.a[cur];
    double* u1 = s.u[cur ^ 1];
    double* v1 = s.v[cur ^ 1];
    double* a1 = s.a[cur ^ 1];
    double rf = 0.0, rff = 0.0;
    bool pending = false;

    if (phase == PH_MIN_STEP) {
        constexpr unsigned SOFT = STEP_SOFT; /* fp64 / integer-pipe split of the step's operations */
        const double uf = sh.uf;
        const Scale skf = I->s_kf;
        double un[PPT], vr[PPT], ar[PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t g = off + l0 + q;
            vr[q] = v0[g];
            ar[q] = a0[g];
            un[q] = S_ADD(3, S_ADD(2, u0[g], S_MUL(0, s.dt, vr[q])), S_MUL(1, s.hdt2, ar[q]));
            sh_un[threadIdx.x * PPT + q] = un[q];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t l = l0 + q;
            if (l >= n) {
                continue;
            }
            int64_t g = off + l;
            double up = un[q];
            double4_32a w = s.wc[g];
            if (!in_well(w.x, w.y, up) && is_nan_bits(up) == false &&
                (__double_as_longlong(up) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL) {
                const double* y = s.data + g * s.W;
                bool ok = false;
                if (y[0] <= up && up < y[s.W - 1]) {
                    int64_t li = s.cidx[g];
                    if (y[li] <= up) {
                        while (li + 1 < s.W && y[li + 1] <= up) {
                            ++li;
                        }
                    }
                    else {
                        while (li > 0 && y[li] > up) {
                            --li;
                        }
                    }
                    if (li >= s.min_margin && li < s.W - s.buffer) {
                        int64_t gold = s.gidx[g];
                        s.cidx[g] = (int32_t)li;
                        s.gidx[g] = s.start[g] + li;
                        w = make_wc(s, y[li], y[li + 1]);
                        s.wc[g] = w;
                        atomicAdd(&sh.ds, (unsigned long long)(s.gidx[g] - gold));
                        ok = true;
                    }
                }
                if (!ok) {
                    pending = true;
                }
            }
            double fp = pot_force<POT_CUSPY, SOFT>(s, w, up);
            double ff = scale(S_SUB(4, uf, up), skf);
            int li2 = threadIdx.x * PPT + q;
            double uL = li2 > 0 ? sh_un[li2 - 1]
                                : (l == 0 ? FQ_ADD(FQ_ADD(u0[off + n - 1], FQ_MUL(s.dt, v0[off + n - 1])),
                                                   FQ_MUL(s.hdt2, a0[off + n - 1]))
                                          : FQ_ADD(FQ_ADD(u0[g - 1], FQ_MUL(s.dt, v0[g - 1])), FQ_MUL(s.hdt2, a0[g - 1])));
            double uR;
            if (li2 + 1 < (int)blockDim.x * PPT && l + 1 < n) {
                uR = sh_un[li2 + 1];
            }
            else {
                int64_t gr = l + 1 == n ? off : g + 1;
                uR = FQ_ADD(FQ_ADD(u0[gr], FQ_MUL(s.dt, v0[gr])), FQ_MUL(s.hdt2, a0[gr]));
            }
            double fi = scale(S_ADD(8, S_SUB(7, uL, scale_pow2(up, 1, 2.0)), uR), s.s_k);
            double sfi = S_ADD(9, S_ADD(6, ff, fp), fi);
            double v = S_ADD(11, vr[q], S_MUL(10, s.dt, ar[q]));
            double f = S_ADD(13, sfi, S_MUL(12, s.me, v));
            double a = scale(f, s.s_im);
            v = S_ADD(16, vr[q], S_MUL(15, s.hdt, S_ADD(14, ar[q], a)));
            f = S_ADD(18, sfi, S_MUL(17, s.me, v));
            a = scale(f, s.s_im);
            v = S_ADD(21, vr[q], S_MUL(20, s.hdt, S_ADD(19, ar[q], a)));
            f = S_ADD(23, sfi, S_MUL(22, s.me, v));
            a = scale(f, s.s_im);
            u1[g] = up;
            v1[g] = v;
            a1[g] = a;
            if (is_nan_bits(up)) {
                sh.nan = 1;
            }
            double f2 = FQ_MUL(f, f), ff2 = FQ_MUL(ff, ff);
            if (q == 0) {
                rf = f2;
                rff = ff2;
            }
            else {
                rf = FQ_ADD(rf, f2);
                rff = FQ_ADD(rff, ff2);
            }
        }
        if (pending && !redo) {
            for (int q = 0; q < PPT; ++q) {
                int64_t l = l0 + q;
                if (l < n) {
                    int64_t g = off + l;
                    double4_32a w = s.wc[g];
                    if (!in_well(w.x, w.y, un[q]) &&
                        (__double_as_longlong(un[q]) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL) {
                        int k = atomicAdd(&b.run->n_regen, 1);
                        b.regen_list[k] = (int32_t)g;
                    }
                }
            }
        }
    }
    else if (phase == PH_EVT_APPLY || phase == PH_KICK_APPLY) {
        const double du = sh.du_p;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t l = l0 + q;
            if (l >= n) {
                continue;
            }
            int64_t g = off + l;
            double x = FQ_ADD(u0[g], du);
            u1[g] = x;
            v1[g] = v0[g];
            a1[g] = a0[g];
            double4_32a w = s.wc[g];
            if (!in_well(w.x, w.y, x) && (__double_as_longlong(x) & 0x7fffffffffffffffLL) < 0x7ff0000000000000LL) {
                const double* y = s.data + g * s.W;
                bool ok = false;
                if (y[0] <= x && x < y[s.W - 1]) {
                    int64_t li = s.cidx[g];
                    if (y[li] <= x) {
                        while (li + 1 < s.W && y[li + 1] <= x) {
                            ++li;
                        }
                    }
                    else {
                        while (li > 0 && y[li] > x) {
                            --li;
                        }
                    }
                    if (li >= s.min_margin && li < s.W - s.buffer) {
                        int64_t gold = s.gidx[g];
                        s.cidx[g] = (int32_t)li;
                        s.gidx[g] = s.start[g] + li;
                        s.wc[g] = make_wc(s, y[li], y[li + 1]);
                        atomicAdd(&sh.ds, (unsigned long long)(s.gidx[g] - gold));
                        ok = true;
                    }
                }
                if (!ok) {
                    pending = true;
                    if (!redo) {
                        int k = atomicAdd(&b.run->n_regen, 1);
                        b.regen_list[k] = (int32_t)g;
                    }
                }
            }
        }
    }
    else if (phase == PH_EVT_MIN) {
        unsigned long long best = 0x7ff0000000000000ULL;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t l = l0 + q;
            if (l < n) {
                int64_t g = off + l;
                double du = FQ_SUB(s.wc[g].y, u0[g]);
                unsigned long long k = (unsigned long long)__double_as_longlong(du);
                best = k < best ? k : best;
            }
        }
        atomicMin(&sh.mkey, best);
    }
    else if (phase == PH_QUENCH) {
        double* vz = s.v[cur];
        double* az = s.a[cur];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t l = l0 + q;
            if (l < n) {
                vz[off + l] = 0.0;
                az[off + l] = 0.0;
            }
        }
    }
    else if (phase == PH_REPORT) {
        const Scale skf = I->s_kf;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            int64_t l = l0 + q;
            double ffq = 0.0;
            if (l < n) {
                ffq = scale(FQ_SUB(sh.uf, u0[off + l]), skf);
            }
            rf = q == 0 ? ffq : FQ_ADD(rf, ffq);
        }
    }
    if (pending && redo) {
        atomicOr(&b.run->walk_flag, 1);
    }
    if (pending && !redo) {
        sh.pending = 1;
    }
    /* tile partials (canonical subtree of the realisation's flat index) */
    bool tree = phase == PH_MIN_STEP || phase == PH_REPORT;
    double sf = 0.0, sff = 0.0;
    if (tree) {
        sf = cta_tree(rf, sh.red);
        __syncthreads();
        sff = cta_tree(rff, sh.red);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (tree) {
            b.partials[t] = make_double2(sf, sff);
        }
        if (sh.ds) {
            atomicAdd((unsigned long long*)&I->s_signed, sh.ds);
        }
        if (phase == PH_EVT_MIN) {
            atomicMin(&I->min_key, sh.mkey);
        }
        if (sh.nan && !sh.pending) {
            atomicOr(&I->nan_flag, 1);
        }
        if (sh.pending) {
            b.tile_pending[t] = 1;
            atomicAdd(&I->n_pending, 1);
            atomicAdd(&b.run->n_pending_tiles, 1);
        }
        __threadfence();
        if (phase != PH_DONE) {
            if (redo) {
                unsigned k = atomicAdd(&I->ticket_redo, 1u);
                sh.last_inst = k == (unsigned)I->n_pending - 1u;
            }
            else {
                unsigned k = atomicAdd(&I->ticket, 1u);
                sh.last_inst = (k == (unsigned)I->ntiles - 1u) && I->n_pending == 0;
                if (k == (unsigned)I->ntiles - 1u && I->n_pending > 0) {
                    I->ticket = 0; /* the redo of this realisation's pending tiles finalises */
                }
            }
        }
    }
    __syncthreads();
    if (sh.last_inst) {
        __threadfence();
        double2 tot = make_double2(0.0, 0.0);
        if (tree) {
            tot = inst_tree(b.partials + I->tile0, I->ntiles, sh.red);
        }
        if (threadIdx.x == 0) {
            inst_finalize(b, I, j, tot);
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (redo) {
            unsigned k = atomicAdd(&b.run->ticket_redo, 1u);
            sh.last_glob = k == (unsigned)b.run->n_pending_tiles - 1u;
        }
        else {
            unsigned k = atomicAdd(&b.run->ticket, 1u);
            sh.last_glob = k == (unsigned)sh.nact - 1u;
        }
    }
    __syncthreads();
    if (sh.last_glob) {
        __threadfence();
        BatchRun* R = b.run;
        const bool iteration_end = redo || R->n_pending_tiles == 0;
        if (iteration_end && R->rebuild) {
            rebuild_active_tiles(b);
        }
        if (threadIdx.x == 0) {
            batch_iteration_end(b, redo != 0);
        }
    }
}

/* the batch's regeneration branch: move the chunk windows recorded by pass 1 (target = new u) */
__global__ void __launch_bounds__(128) k_batch_regen(BatchDev b)
{
    const int nreg = b.run->n_regen;
    const DevSys& s = b.d;
    if (nreg >= (int)(gridDim.x * blockDim.x) / 4) {
        /* many moves: one thread per particle */
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nreg; k += gridDim.x * blockDim.x) {
            int64_t g = b.regen_list[k];
            int j = b.tile_inst[g / b.tile];
            Inst* I = b.inst + j;
            double x = s.u[I->cur ^ 1][g];
            int64_t gold = s.gidx[g];
            if (!dev_align(s, g, x)) {
                atomicOr(&b.run->walk_flag, 1);
            }
            atomicAdd((unsigned long long*)&I->s_signed, (unsigned long long)(s.gidx[g] - gold));
        }
        return;
    }
    /* few moves: one CTA per particle, its threads sharing the draws (fwd_move_*); the same values */
    __shared__ FwdMove m_sh;
    __shared__ int ok_sh;
    __shared__ long long gold_sh;
    const uint64_t mv_c = pcg_advance(0ULL, (uint64_t)blockDim.x);
    const uint64_t mv_a = pcg_advance(1ULL, (uint64_t)blockDim.x) - mv_c;
    for (int k = blockIdx.x; k < nreg; k += gridDim.x) {
        const int64_t g = b.regen_list[k];
        Inst* I = b.inst + b.tile_inst[g / b.tile];
        if (threadIdx.x == 0) {
            double x = s.u[I->cur ^ 1][g];
            gold_sh = s.gidx[g];
            FwdMove m;
            ok_sh = fwd_move_plan(s, g, x, m) ? 1 : 0;
            if (ok_sh) {
                m_sh = m;
            }
            else if (!dev_align(s, g, x)) {
                atomicOr(&b.run->walk_flag, 1);
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
            atomicAdd((unsigned long long*)&I->s_signed, (unsigned long long)(s.gidx[g] - gold_sh));
        }
        __syncthreads();
    }
}

/* initial chunk windows [0, W) and wells at u = 0 */
__global__ void k_batch_init(DevSys d, const int64_t* owner_valid)
{
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= d.N || !owner_valid[g]) {
        return;
    }
    d.anc_kind[g] = 0;
    double* y = d.data + g * d.W;
    double acc;
    seq_fill(d, g, 0, d.W, y, &acc);
    d.start[g] = 0;
    d.cidx[g] = 0;
    d.gidx[g] = 0;
    d.acc_end[g] = acc;
    d.wc[g] = make_wc(d, y[0], y[1]);
    dev_align(d, g, 0.0);
}

static cudaError_t add_kernel_node(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t nd,
                                   void* func, dim3 grid, dim3 block, void** args)
{
    cudaKernelNodeParams kp = {};
    kp.func = func;
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.kernelParams = args;
    return cudaGraphAddKernelNode(node, graph, deps, nd, &kp);
}

static cudaError_t add_cond(cudaGraphNode_t* node, cudaGraph_t graph, const cudaGraphNode_t* deps, size_t nd,
                            cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type, cudaGraph_t* body)
{
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaError_t e = cudaGraphAddNode(node, graph, deps, nullptr, nd, &np);
    if (e == cudaSuccess) {
        *body = np.conditional.phGraph_out[0];
    }
    return e;
}

static cudaError_t build_batch_graph(BatchDev& b, int threads, cudaGraphExec_t* exec)
{
    cudaGraph_t g;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess) {
        return e;
    }
#define BG(expr)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (expr);                                                                       \
        if (e_ != cudaSuccess) {                                                                       \
            cudaGraphDestroy(g);                                                                       \
            return e_;                                                                                 \
        }                                                                                              \
    } while (0)
    cudaGraphConditionalHandle hw, hi;
    BG(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t wn;
    cudaGraph_t body;
    BG(add_cond(&wn, g, nullptr, 0, hw, cudaGraphCondTypeWhile, &body));
    BG(cudaGraphConditionalHandleCreate(&hi, body, 0, cudaGraphCondAssignDefault));
    b.h_while = hw;
    b.h_if = hi;
    b.in_graph = 1;
    void* fk = b.ppt == 2 ? (void*)k_batch<2> : (void*)k_batch<1>;
    int pass1 = 0, pass2 = 1;
    void* a1[] = {(void*)&b, (void*)&pass1};
    void* a2[] = {(void*)&b, (void*)&pass2};
    void* ar[] = {(void*)&b};
    cudaGraphNode_t ns, nif, nr, nd;
    BG(add_kernel_node(&ns, body, nullptr, 0, fk, dim3((unsigned)b.ntiles), dim3((unsigned)threads), a1));
    cudaGraph_t ifb;
    BG(add_cond(&nif, body, &ns, 1, hi, cudaGraphCondTypeIf, &ifb));
    BG(add_kernel_node(&nr, ifb, nullptr, 0, (void*)k_batch_regen, dim3(4 * 152), dim3(128), ar));
    BG(add_kernel_node(&nd, ifb, &nr, 1, fk, dim3((unsigned)b.ntiles), dim3((unsigned)threads), a2));
#undef BG
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    return e;
}

} // namespace fqsb

using namespace fqsb;

struct fqsb_batch {
    BatchDev b;
    int64_t ninst, nchunk, window;
    int threads, ppt;
    std::vector<int64_t> sizes, offs;
    std::vector<double> kframe;
    cudaStream_t stream;
    bool own_stream;
    bool no_graph; /* FQSB_NO_GRAPH=1 at creation: passes launched one by one (for profilers) */
    cudaGraphExec_t graph;
    std::string err;
    std::vector<void*> allocs;
};

static std::string g_batch_error;

static int berr(fqsb_batch* h, int code, const std::string& m)
{
    if (h) {
        h->err = m;
    }
    else {
        g_batch_error = m;
    }
    return code;
}

#define BCU(h, expr)                                                                                     \
    do {                                                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            return berr((h), FQSB_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_));           \
        }                                                                                                \
    } while (0)

static Scale classify(double c)
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

extern "C" const char* fqsb_batch_last_error(const fqsb_batch* h)
{
    return h ? h->err.c_str() : g_batch_error.c_str();
}

static void batch_free(fqsb_batch* h)
{
    if (!h) {
        return;
    }
    for (void* p : h->allocs) {
        cudaFree(p);
    }
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
    }
    if (h->own_stream && h->stream) {
        cudaStreamDestroy(h->stream);
    }
    delete h;
}

template <class T>
static cudaError_t balloc(fqsb_batch* h, T** p, size_t count)
{
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) {
        h->allocs.push_back((void*)*p);
    }
    return e;
}

extern "C" int fqsb_batch_create(const fqsb_batch_config* c, fqsb_batch** out)
{
    FQSB_API_RANGE();
    if (!c || !out || c->n_instances < 1 || !c->sizes || !c->seeds || !c->k_frame) {
        return berr(nullptr, FQSB_ERR_INVALID, "invalid batch configuration");
    }
    if (c->nchunk < 34 || c->window < 34 || c->window > c->nchunk || c->n_parameters < 0 || c->n_parameters > 4) {
        return berr(nullptr, FQSB_ERR_INVALID, "need 34 <= window <= nchunk and at most 4 parameters");
    }
    /* default tile: 256 threads x 2 particles (measured fastest of the autotuner's candidates on a
     * log-uniform [256, 65536] batch: 15.6 G particle-steps/s against 11.6 for 256 x 1) */
    int threads = c->threads ? c->threads : 256;
    int ppt = c->ppt ? c->ppt : 2;
    if (!(threads == 32 || threads == 64 || threads == 128 || threads == 256) || !(ppt == 1 || ppt == 2)) {
        return berr(nullptr, FQSB_ERR_INVALID, "threads must be 32, 64, 128 or 256 and ppt 1 or 2");
    }
    int dist = c->distribution;
    if (!(dist == FQSB_DIST_RANDOM || dist == FQSB_DIST_DELTA || dist == FQSB_DIST_EXPONENTIAL ||
          dist == FQSB_DIST_POWER || dist == FQSB_DIST_PARETO || dist == FQSB_DIST_WEIBULL)) {
        return berr(nullptr, FQSB_ERR_UNSUPPORTED, "distribution not supported");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return berr(nullptr, FQSB_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (cudaSetDevice(c->device) != cudaSuccess) {
        return berr(nullptr, FQSB_ERR_NO_DEVICE, "cudaSetDevice failed");
    }
    fqsb_batch* h = new fqsb_batch();
    h->graph = nullptr;
    {
        const char* ng = getenv("FQSB_NO_GRAPH");
        h->no_graph = ng && ng[0] == '1';
    }
    h->ninst = c->n_instances;
    h->nchunk = c->nchunk;
    h->window = c->window;
    h->threads = threads;
    h->ppt = ppt;
    if (c->stream) {
        h->stream = (cudaStream_t)c->stream;
        h->own_stream = false;
    }
    else {
        cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
        h->own_stream = true;
    }
    int tile = threads * ppt;
    std::vector<int32_t> tile_inst;
    std::vector<Inst> inst((size_t)h->ninst);
    int64_t total = 0;
    for (int64_t j = 0; j < h->ninst; ++j) {
        int64_t n = c->sizes[j];
        if (n < 3) {
            batch_free(h);
            return berr(nullptr, FQSB_ERR_INVALID, "each realisation needs at least 3 particles");
        }
        int64_t nt = (n + tile - 1) / tile;
        Inst& I = inst[(size_t)j];
        memset(&I, 0, sizeof(Inst));
        I.off = total;
        I.n = n;
        I.tile0 = (int64_t)tile_inst.size();
        I.ntiles = nt;
        I.k_frame = c->k_frame[j];
        I.s_kf = classify(c->k_frame[j]);
        I.u_frame = 0.0;
        I.phase = PH_EVT_MIN;
        I.min_key = 0x7ff0000000000000ULL;
        for (int64_t k = 0; k < nt; ++k) {
            tile_inst.push_back((int32_t)j);
        }
        h->sizes.push_back(n);
        h->offs.push_back(total);
        h->kframe.push_back(c->k_frame[j]);
        total += nt * tile;
    }
    if (total >= ((int64_t)1 << 31)) {
        batch_free(h);
        return berr(nullptr, FQSB_ERR_INVALID, "too many particles in one batch (>= 2^31 with padding)");
    }
    BatchDev& b = h->b;
    memset(&b, 0, sizeof(BatchDev));
    DevSys& d = b.d;
    d.N = total;
    d.rows = 1;
    d.cols = total;
    d.pot = POT_CUSPY;
    d.inter = INTER_LAPLACE1D;
    d.dt = c->dt;
    d.hdt = 0.5 * c->dt;
    d.hdt2 = 0.5 * c->dt * c->dt;
    d.mu = c->mu;
    d.k = c->k_interactions;
    d.me = -c->eta;
    d.m = c->m;
    d.inv_m = 1.0 / c->m;
    d.s_mu = classify(d.mu);
    d.s_k = classify(d.k);
    d.s_kf = classify(1.0);
    d.s_im = classify(d.inv_m);
    d.W = c->window;
    d.n0 = c->nchunk;
    d.dist = dist;
    d.npar = c->n_parameters;
    for (int i = 0; i < 4; ++i) {
        d.par[i] = i < c->n_parameters ? c->parameters[i] : 0.0;
    }
    d.offset = c->offset;
    d.buffer = 2;
    d.margin = 30;
    d.min_margin = 6;
    b.ntiles = (int64_t)tile_inst.size();
    b.tile = tile;
    b.ppt = ppt;
    size_t N = (size_t)total;
    std::vector<uint64_t> pseed(N, 0);
    std::vector<int64_t> valid(N, 0);
    for (int64_t j = 0; j < h->ninst; ++j) {
        for (int64_t l = 0; l < c->sizes[j]; ++l) {
            pseed[(size_t)(h->offs[(size_t)j] + l)] = c->seeds[j] + (uint64_t)l;
            valid[(size_t)(h->offs[(size_t)j] + l)] = 1;
        }
    }
#define BA(p, cnt)                                                                                       \
    do {                                                                                                 \
        cudaError_t e_ = balloc(h, &(p), (cnt));                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            std::string m_ = std::string("device allocation failed: ") + cudaGetErrorString(e_);         \
            batch_free(h);                                                                               \
            return berr(nullptr, FQSB_ERR_CUDA, m_);                                                     \
        }                                                                                                \
    } while (0)
    double* data;
    BA(data, N * (size_t)d.W);
    d.data = data;
    BA(d.start, N);
    BA(d.cidx, N);
    BA(d.gidx, N);
    BA(d.wc, N);
    BA(d.acc_end, N);
    BA(d.anc_kind, N);
    BA(d.anc_k, N);
    BA(d.anc_state, N);
    BA(d.anc_val, N);
    uint64_t* ps;
    BA(ps, N);
    d.pseed = ps;
    for (int k = 0; k < 2; ++k) {
        BA(d.u[k], N);
        BA(d.v[k], N);
        BA(d.a[k], N);
    }
    Ctl* ctl;
    BA(ctl, 1);
    d.ctl = ctl;
    BA(b.inst, (size_t)h->ninst);
    BA(b.run, 1);
    int32_t* ti;
    BA(ti, (size_t)b.ntiles);
    b.tile_inst = ti;
    BA(b.partials, (size_t)b.ntiles);
    BA(b.tile_pending, (size_t)b.ntiles);
    BA(b.active_tiles, (size_t)b.ntiles);
    b.ninst = h->ninst;
    BA(b.regen_list, N);
    int64_t* dvalid;
    BA(dvalid, N);
#undef BA
    cudaStream_t st = h->stream;
    bool ok = cudaMemcpyAsync(ps, pseed.data(), sizeof(uint64_t) * N, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(dvalid, valid.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ti, tile_inst.data(), sizeof(int32_t) * tile_inst.size(), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemcpyAsync(b.inst, inst.data(), sizeof(Inst) * inst.size(), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemsetAsync(b.run, 0, sizeof(BatchRun), st) == cudaSuccess &&
              cudaMemsetAsync(b.tile_pending, 0, sizeof(int32_t) * (size_t)b.ntiles, st) == cudaSuccess &&
              cudaMemsetAsync(ctl, 0, sizeof(Ctl), st) == cudaSuccess;
    for (int k = 0; k < 2 && ok; ++k) {
        ok = cudaMemsetAsync(d.u[k], 0, sizeof(double) * N, st) == cudaSuccess &&
             cudaMemsetAsync(d.v[k], 0, sizeof(double) * N, st) == cudaSuccess &&
             cudaMemsetAsync(d.a[k], 0, sizeof(double) * N, st) == cudaSuccess;
    }
    if (!ok) {
        batch_free(h);
        return berr(nullptr, FQSB_ERR_CUDA, "batch initialisation copies failed");
    }
    k_batch_init<<<(unsigned)((N + 63) / 64), 64, 0, st>>>(d, dvalid);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) {
        std::string m = std::string("batch construction failed: ") + cudaGetErrorString(e);
        batch_free(h);
        return berr(nullptr, FQSB_ERR_CUDA, m);
    }
    e = build_batch_graph(b, threads, &h->graph);
    if (e != cudaSuccess) {
        std::string m = std::string("batch graph: ") + cudaGetErrorString(e);
        batch_free(h);
        return berr(nullptr, FQSB_ERR_CUDA, m);
    }
    *out = h;
    return FQSB_OK;
}

extern "C" int fqsb_batch_destroy(fqsb_batch* h)
{
    if (h) {
        cudaStreamSynchronize(h->stream);
        batch_free(h);
    }
    return FQSB_OK;
}

extern "C" int fqsb_batch_quasistatic(fqsb_batch* h, int64_t ncycles, double eps, double tol, uint64_t niter_tol,
                                      uint64_t max_iter, double* u_frame_out, double* f_frame_out, int64_t* S_out,
                                      int64_t* inc_out, int32_t* status_out)
{
    FQSB_API_RANGE();
    if (!h || ncycles < 1 || !u_frame_out || !f_frame_out || !S_out || !inc_out || !status_out) {
        return FQSB_ERR_INVALID;
    }
    if (niter_tol > (uint64_t)BATCH_RING) {
        return berr(h, FQSB_ERR_INVALID, "niter_tol must be <= 64 in the batched form");
    }
    if (!(tol < 1.0)) {
        return berr(h, FQSB_ERR_INVALID, "assertion failed (tol < 1.0)");
    }
    if (ncycles > (int64_t)INT32_MAX || (uint64_t)h->ninst > (SIZE_MAX / sizeof(double)) / (uint64_t)ncycles) {
        return berr(h, FQSB_ERR_INVALID, "ncycles too large");
    }
    BatchDev& b = h->b;
    const size_t nout = (size_t)h->ninst * (size_t)ncycles;
    double *du = nullptr, *df = nullptr;
    int64_t *dS = nullptr, *dI = nullptr;
    /* one exit path for every outcome: the output buffers are freed, and the graph (whose kernel
     * arguments point at them) is destroyed with the pointers cleared */
    auto release = [&]() {
        for (void* p : {(void*)du, (void*)df, (void*)dS, (void*)dI}) {
            if (p) {
                cudaFree(p);
            }
        }
        b.out_uframe = nullptr;
        b.out_fframe = nullptr;
        b.out_S = nullptr;
        b.out_inc = nullptr;
        if (h->graph) {
            cudaGraphExecDestroy(h->graph);
            h->graph = nullptr;
        }
    };
#define QCU(expr)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (expr);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            release();                                                                                   \
            return berr(h, FQSB_ERR_CUDA, std::string(#expr ": ") + cudaGetErrorString(e_));             \
        }                                                                                                \
    } while (0)
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    QCU(cudaMalloc(&du, sizeof(double) * nout));
    QCU(cudaMalloc(&df, sizeof(double) * nout));
    QCU(cudaMalloc(&dS, sizeof(int64_t) * nout));
    QCU(cudaMalloc(&dI, sizeof(int64_t) * nout));
    b.out_uframe = du;
    b.out_fframe = df;
    b.out_S = dS;
    b.out_inc = dI;
    /* the output pointers are kernel arguments: build the graph for this run */
    QCU(build_batch_graph(b, h->threads, &h->graph));
    /* reset every realisation's protocol state (keeps u, v, a, wells and frame positions) */
    std::vector<Inst> inst((size_t)h->ninst);
    QCU(cudaMemcpy(inst.data(), b.inst, sizeof(Inst) * inst.size(), cudaMemcpyDeviceToHost));
    for (auto& I : inst) {
        I.phase = PH_EVT_MIN;
        I.cycle = 0;
        I.status = BST_OK;
        I.ticket = I.ticket_redo = 0;
        I.n_pending = 0;
        I.nan_flag = 0;
        I.s_signed = 0;
        I.min_key = 0x7ff0000000000000ULL;
    }
    QCU(cudaMemcpyAsync(b.inst, inst.data(), sizeof(Inst) * inst.size(), cudaMemcpyHostToDevice, h->stream));
    BatchRun R;
    memset(&R, 0, sizeof(R));
    R.ncycles = (int32_t)ncycles;
    R.niter_tol = (int32_t)niter_tol;
    R.eps = eps;
    R.tol = tol;
    R.tol2 = tol * tol;
    R.max_iter = (int64_t)max_iter;
    R.active = (int32_t)h->ninst;
    R.budget_ns = 200ull * 1000ull * 1000ull;
    /* every realisation starts the protocol: all tiles are active */
    R.n_active_tiles = (int32_t)b.ntiles;
    R.rebuild = 0;
    {
        std::vector<int32_t> all((size_t)b.ntiles);
        for (size_t k = 0; k < all.size(); ++k) {
            all[k] = (int32_t)k;
        }
        QCU(cudaMemcpy(b.active_tiles, all.data(), sizeof(int32_t) * all.size(), cudaMemcpyHostToDevice));
    }
    QCU(cudaMemcpyAsync(b.run, &R, sizeof(R), cudaMemcpyHostToDevice, h->stream));
    if (h->no_graph) {
        /* each pass launched by the host: pass 1, and the regeneration branch when tiles are pending */
        BatchDev bh = b;
        bh.in_graph = 0;
        void* fk = b.ppt == 2 ? (void*)k_batch<2> : (void*)k_batch<1>;
        int pass1 = 0, pass2 = 1;
        void* a1[] = {(void*)&bh, (void*)&pass1};
        void* a2[] = {(void*)&bh, (void*)&pass2};
        void* ar[] = {(void*)&bh};
        for (;;) {
            QCU(cudaLaunchKernel(fk, dim3((unsigned)b.ntiles), dim3((unsigned)h->threads), a1, 0, h->stream));
            QCU(cudaMemcpyAsync(&R, b.run, sizeof(R), cudaMemcpyDeviceToHost, h->stream));
            QCU(cudaStreamSynchronize(h->stream));
            if (R.n_pending_tiles > 0) {
                QCU(cudaLaunchKernel((void*)k_batch_regen, dim3(4 * 152), dim3(128), ar, 0, h->stream));
                QCU(cudaLaunchKernel(fk, dim3((unsigned)b.ntiles), dim3((unsigned)h->threads), a2, 0, h->stream));
                QCU(cudaMemcpyAsync(&R, b.run, sizeof(R), cudaMemcpyDeviceToHost, h->stream));
                QCU(cudaStreamSynchronize(h->stream));
            }
            if (R.active <= 0 || R.walk_flag) {
                break;
            }
        }
    }
    else {
        for (;;) {
            QCU(cudaGraphLaunch(h->graph, h->stream));
            QCU(cudaMemcpyAsync(&R, b.run, sizeof(R), cudaMemcpyDeviceToHost, h->stream));
            QCU(cudaStreamSynchronize(h->stream));
            if (R.active <= 0 || R.walk_flag) {
                break;
            }
            int64_t zero = 0;
            QCU(cudaMemcpyAsync(&b.run->launch_iters, &zero, sizeof(zero), cudaMemcpyHostToDevice, h->stream));
        }
    }
    QCU(cudaMemcpy(u_frame_out, du, sizeof(double) * nout, cudaMemcpyDeviceToHost));
    QCU(cudaMemcpy(f_frame_out, df, sizeof(double) * nout, cudaMemcpyDeviceToHost));
    QCU(cudaMemcpy(S_out, dS, sizeof(int64_t) * nout, cudaMemcpyDeviceToHost));
    QCU(cudaMemcpy(inc_out, dI, sizeof(int64_t) * nout, cudaMemcpyDeviceToHost));
    QCU(cudaMemcpy(inst.data(), b.inst, sizeof(Inst) * inst.size(), cudaMemcpyDeviceToHost));
#undef QCU
    release();
    for (size_t j = 0; j < inst.size(); ++j) {
        status_out[j] = inst[j].status;
    }
    if (R.walk_flag) {
        return berr(h, FQSB_ERR_TIMEOUT, "yield search exceeded its bound");
    }
    return FQSB_OK;
}

extern "C" int fqsb_batch_get(fqsb_batch* h, int64_t instance, int field, double* out)
{
    if (!h || !out || instance < 0 || instance >= h->ninst) {
        return FQSB_ERR_INVALID;
    }
    Inst I;
    BCU(h, cudaMemcpy(&I, h->b.inst + instance, sizeof(Inst), cudaMemcpyDeviceToHost));
    const double* src;
    if (field == FQSB_FIELD_U) {
        src = h->b.d.u[I.cur];
    }
    else if (field == FQSB_FIELD_V) {
        src = h->b.d.v[I.cur];
    }
    else if (field == FQSB_FIELD_A) {
        src = h->b.d.a[I.cur];
    }
    else {
        return berr(h, FQSB_ERR_INVALID, "field must be u, v or a");
    }
    BCU(h, cudaMemcpy(out, src + I.off, sizeof(double) * (size_t)I.n, cudaMemcpyDeviceToHost));
    return FQSB_OK;
}

extern "C" int fqsb_batch_get_index(fqsb_batch* h, int64_t instance, int64_t* out)
{
    if (!h || !out || instance < 0 || instance >= h->ninst) {
        return FQSB_ERR_INVALID;
    }
    int64_t off = h->offs[(size_t)instance], n = h->sizes[(size_t)instance];
    BCU(h, cudaMemcpy(out, h->b.d.gidx + off, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost));
    return FQSB_OK;
}

extern "C" int fqsb_batch_frame(fqsb_batch* h, double* u_frame)
{
    if (!h || !u_frame) {
        return FQSB_ERR_INVALID;
    }
    std::vector<Inst> inst((size_t)h->ninst);
    BCU(h, cudaMemcpy(inst.data(), h->b.inst, sizeof(Inst) * inst.size(), cudaMemcpyDeviceToHost));
    for (size_t j = 0; j < inst.size(); ++j) {
        u_frame[j] = inst[j].u_frame;
    }
    return FQSB_OK;
}
