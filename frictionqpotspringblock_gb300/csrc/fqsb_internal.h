/*
 * Internal host-side interface between the C-ABI layer (fqsb_capi.cu) and the
 * kernel translation units.  Not installed; the public ABI is include/fqsb.h.
 */
#ifndef FQSB_INTERNAL_H
#define FQSB_INTERNAL_H

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>

#include <string>

#include "fqsb_device.cuh"

namespace fqsb {

/* Launch geometry of the 1d step kernel: threads per CTA and particles per thread. */
struct LineGeom {
    int threads;
    int ppt;
    int64_t grid;
};

LineGeom line_geometry(int64_t N);

/* Message returned by fqsb_last_error(NULL) (errors of calls that have no handle). */
void set_global_error(const std::string& msg);

/* Per-particle canonical reduction of the step's residual terms (used by the 2d path). */
int64_t grid_reduce_ctas(int64_t N);

/* Number of CTAs of the step kernel (size of DevSys::cta_pending and DevSys::partials). */
int64_t step_ctas(const DevSys& s, const LineGeom& g);

/* The run graph: a device-side WHILE loop over fused steps, with the chunk-regeneration branch.
 * Writes the conditional handles into s (they are kernel arguments of the graph's nodes). */
/* Step-kernel instantiations: the general one, and for athermal Line1d / Particles systems two
 * specialised ones -- runs without activity, residual, frame-force sums or recording (timeSteps /
 * flowSteps), and runs with the residual only (minimise) -- with the other code compiled out. */
enum : int { KMODE_GENERAL = 0, KMODE_PLAIN = 1, KMODE_RESID = 2 };
cudaError_t build_run_graph(DevSys& s, const LineGeom& g, cudaGraphExec_t* exec, int mode = KMODE_GENERAL);
/* Whether the system has the specialised step kernels (athermal Line1d / Particles systems). */
bool plain_runs_apply(const DevSys& s);

/* Small Line1d / Particles systems: a whole run in one launch of one thread-block cluster. */
static const int SMALL_MAX_CTAS = 16;   /* cluster size limit (above 8 needs the non-portable opt-in) */
static const int SMALL_RING_MAX = 1024; /* StopList windows up to this length stay in shared memory */
/* small systems keep a next-window buffer (N x nchunk doubles) up to this many values */
static const int64_t NX_MAX_VALUES = (int64_t)1 << 25;
static const int SMALL_THREADS_MAX = 256; /* particle threads per CTA (each CTA adds one control warp) */
struct SmallGeom {
    int threads; /* per CTA, power of two in [32, 256] */
    int ppt;     /* particles per thread: 1, 2 or 4 */
    int ctas;    /* CTAs of the cluster */
    bool ok;     /* N fits: N <= max_ctas * 1024 */
};
SmallGeom small_geometry(int64_t N, int max_ctas);
cudaError_t launch_small_run(const DevSys& s, const SmallGeom& g, cudaStream_t st);
/* refreshes the next-window buffers of a small system (no-op when it has none) */
cudaError_t launch_next_window(const DevSys& s, cudaStream_t st);
/* Whether a cluster of g.ctas CTAs of this kernel can be co-scheduled (sizes above 8 are opt-in). */
bool small_cluster_fits(const DevSys& s, const SmallGeom& g);

/* Arguments of the no-passing minimiser's kernels (the force arrays are the handle's stored forces). */
struct NopassArgs {
    double *f_pot, *f_int, *f_frame, *f;
    double den; /* (2 k + k_frame) + mu */
    int ppt;    /* particles per thread (the step's launch shape, for the canonical residual tree) */
};
static const int NOPASS_MAX_REALIGN = 1 << 20; /* bound on one particle's well updates in one sweep */
cudaError_t build_nopass_graph(const DevSys& s, const LineGeom& g, const NopassArgs& A, cudaGraphExec_t* exec);
cudaError_t launch_nopass_iteration(const DevSys& s, const LineGeom& g, const NopassArgs& A, cudaStream_t st);

/* RandomNormalForcing draw (updated_inc): from_ctl = 1 for the step a run is about to make (inside
 * the run loop), else at increment `inc`.  thermal_tiles: size of DevSys::th_cnt. */
cudaError_t launch_thermal_draw(const DevSys& s, int from_ctl, int64_t inc, cudaStream_t st);
int64_t thermal_tiles(int64_t N);

/* One loop iteration launched kernel by kernel by the host (s.in_graph must be 0). */
cudaError_t launch_iteration(const DevSys& s, const LineGeom& g, cudaStream_t st, int mode = KMODE_GENERAL);

/* NVTX range over one C-ABI call: each stepping / construction call shows as a named range on a
 * profiler timeline (header-only NVTX 3; a no-op unless a tool is attached). */
struct ApiRange {
    explicit ApiRange(const char* name)
    {
        nvtxRangePushA(name);
    }
    ~ApiRange()
    {
        nvtxRangePop();
    }
    ApiRange(const ApiRange&) = delete;
    ApiRange& operator=(const ApiRange&) = delete;
};
#define FQSB_API_RANGE() fqsb::ApiRange fqsb_api_range_(__func__)

/* Arguments of one backward step of the adjoint (fqsb_adjoint.cu). */
struct AdjArgs {
    const double *u_in, *v_in, *a_in; /* input state of the step */
    const double* up;                 /* output positions of the step */
    const double4_32a* w;             /* wells used by the step */
    double uf;                        /* u_frame of the step */
    double wff;                       /* dL / d f_frame[p] of the step (loss window) */
    const double *lu_out, *lv_out, *la_out;
    double *lu_in, *lv_in, *la_in;
    double4_32a* partials; /* per CTA */
    double* step_out;      /* 4 doubles: sum k_frame dL/df_frame, dL/deta, dL/dmu, dL/dk of the step */
    unsigned* ticket;
};

cudaError_t launch_adjoint_step(const DevSys& s, const AdjArgs& A, cudaStream_t st);
int64_t adjoint_ctas(int64_t N);

} // namespace fqsb

#endif
