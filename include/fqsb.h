/*
 * fqsb.h -- C ABI of the GB300-native FrictionQPotSpringBlock time-integration path.
 *
 * One opaque handle owns one system (a Line1d / Line2d / Particles System_*
 * of the reference) resident in device memory.  Every entry point is
 * synchronous at return, takes plain pointers and sizes (host memory unless
 * the name ends in _device), and returns an fqsb_status; the message of the
 * last failure is available from fqsb_last_error().  Error texts reproduce
 * the reference's exceptions ("NaN entries found", "No convergence found",
 * "Operation not possible.").
 *
 * Each declaration names the reference interface it replaces, as
 * file:line inside the reference project (python/main.cpp is the pybind11
 * boundary; include/FrictionQPotSpringBlock/detail.h holds the C++ methods).
 */
#ifndef FQSB_H
#define FQSB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fqsb_system fqsb_system;

typedef enum {
    FQSB_OK = 0,
    FQSB_ERR_NAN = 1,            /* "NaN entries found"          detail.h:1567-1569 */
    FQSB_ERR_NO_CONVERGENCE = 2, /* "No convergence found"       detail.h:1787-1789 */
    FQSB_ERR_INVALID = 3,        /* invalid argument / shape */
    FQSB_ERR_CUDA = 4,           /* CUDA runtime error */
    FQSB_ERR_TIMEOUT = 5,        /* a bounded device wait ran out */
    FQSB_ERR_NOT_POSSIBLE = 6,   /* "Operation not possible."    detail.h:414-422 */
    FQSB_ERR_REQUIRE = 7,        /* FRICTIONQPOTSPRINGBLOCK_REQUIRE failed, detail.h:1992-1994 */
    FQSB_ERR_UNSUPPORTED = 8,    /* distribution not implemented on the device */
    FQSB_ERR_NO_DEVICE = 9       /* no CUDA device available */
} fqsb_status;

/* potential (detail.h:113 Cuspy, :212 SemiSmooth, :356 Smooth) */
enum { FQSB_CUSPY = 0, FQSB_SEMISMOOTH = 1, FQSB_SMOOTH = 2 };
/* interactions (none = Particles.h:93-311; detail.h:446 Laplace1d; :524 Laplace2d) */
enum {
    FQSB_INTERACTIONS_NONE = 0,
    FQSB_LAPLACE1D = 1,          /* detail.h:446-488 */
    FQSB_LAPLACE2D = 2,          /* detail.h:524-584 */
    FQSB_QUARTIC1D = 3,          /* detail.h:757-805, Line1d.System_Cuspy_Quartic (main.cpp:768-810) */
    FQSB_QUARTICGRADIENT1D = 4,  /* detail.h:616-653, Line1d.System_Cuspy_QuarticGradient (main.cpp:813-855) */
    FQSB_QUARTICGRADIENT2D = 5,  /* detail.h:658-751, Line2d.System_Cuspy_QuarticGradient (main.cpp:963-1005) */
    FQSB_LONGRANGE1D = 6         /* detail.h:812-868, Line1d.System_Cuspy_LongRange (main.cpp:857-897) */
};
/* distributions, prrng names (detail.h:31-66) */
enum {
    FQSB_DIST_RANDOM = 0,
    FQSB_DIST_DELTA = 1,
    FQSB_DIST_EXPONENTIAL = 2,
    FQSB_DIST_POWER = 3,
    FQSB_DIST_GAMMA = 4,
    FQSB_DIST_PARETO = 5,
    FQSB_DIST_WEIBULL = 6,
    FQSB_DIST_NORMAL = 7
};
/* per-particle fields (main.cpp:80-127) */
enum {
    FQSB_FIELD_U = 0,
    FQSB_FIELD_V = 1,
    FQSB_FIELD_A = 2,
    FQSB_FIELD_F = 3,
    FQSB_FIELD_F_POTENTIAL = 4,
    FQSB_FIELD_F_INTERACTIONS = 5,
    FQSB_FIELD_F_FRAME = 6,
    FQSB_FIELD_F_DAMPING = 7
};
/* scalars */
enum {
    FQSB_SCALAR_U_FRAME = 0,     /* main.cpp:104 */
    FQSB_SCALAR_T = 1,           /* main.cpp:103 */
    FQSB_SCALAR_TEMPERATURE = 2, /* main.cpp:128, detail.h:1500-1503 */
    FQSB_SCALAR_RESIDUAL = 3,    /* main.cpp:129, detail.h:1512-1520 */
    FQSB_SCALAR_MEAN_F_FRAME = 4 /* xt::mean(f_frame), detail.h:1991 */
};

/*
 * Construction parameters.  Replaces the constructors
 *   Line1d::System_Cuspy_Laplace       main.cpp:493-520, Line1d.h:134-161
 *   Line1d::System_SemiSmooth_Laplace  main.cpp:684-713, Line1d.h:348-376
 *   Line1d::System_Smooth_Laplace      main.cpp:729-756, Line1d.h:394-421
 *   Line2d::System_Cuspy_Laplace       main.cpp:924-951, Line2d.h:88-115
 *   Particles::System_{Cuspy,SemiSmooth,Smooth}  Particles.h:93-311
 */
typedef struct {
    int potential;           /* FQSB_CUSPY / FQSB_SEMISMOOTH / FQSB_SMOOTH */
    int interactions;        /* FQSB_INTERACTIONS_NONE / FQSB_LAPLACE1D / FQSB_LAPLACE2D / FQSB_QUARTIC* */
    int64_t rows, cols;      /* 1d: rows = 1, cols = N */
    double m, eta, mu, kappa, k_interactions, k_frame, dt;
    uint64_t seed;           /* particle p uses pcg32(initstate = seed + p, initseq = 0) */
    int distribution;        /* FQSB_DIST_* */
    int n_parameters;        /* <= 4 */
    double parameters[4];
    double offset;           /* global shift of the yield positions (Line1d.h:157) */
    const double* offset_per_particle; /* extension, may be NULL: per-particle shift replacing `offset` */
    int64_t nchunk;          /* yield positions held per particle (>= 34) */
    void* stream;            /* cudaStream_t to run on, or NULL for a private stream */
    int device;              /* CUDA device ordinal */
    double interaction_parameters[2]; /* Quartic1d: a1, a2; QuarticGradient1d / 2d: k2, k4; LongRange1d: alpha
                                         (with k_interactions); Laplace: unused */
} fqsb_config;

/* Lifecycle. */
int fqsb_create(const fqsb_config* cfg, fqsb_system** out);
int fqsb_destroy(fqsb_system* h);
const char* fqsb_last_error(const fqsb_system* h); /* h may be NULL: last error of fqsb_create */
int fqsb_size(const fqsb_system* h, int64_t* n);

/* Dynamics. */
int fqsb_time_step(fqsb_system* h);                               /* timeStep         main.cpp:212, detail.h:1539 */
int fqsb_time_steps(fqsb_system* h, uint64_t n);                  /* timeSteps        main.cpp:213, detail.h:1577 */
int fqsb_flow_steps(fqsb_system* h, uint64_t n, double v_frame);  /* flowSteps        main.cpp:224, detail.h:1637 */
int fqsb_time_steps_until_event(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter,
                                uint64_t* ret);                    /* timeStepsUntilEvent main.cpp:215-222, detail.h:1595 */
int fqsb_minimise(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                  int max_iter_is_error, uint64_t* ret);           /* minimise         main.cpp:161-170, detail.h:1676 */
/* minimise of Line1d.System_Cuspy_Laplace_Nopassing: the overdamped no-passing fixed point (Jacobi sweeps),
 * main.cpp:532-568 (class), detail.h:1694-1753 (the Overdamped branch of minimise).  Cuspy + Laplace1d,
 * N >= 2; inc does not advance; on convergence v = a = 0 (quench), otherwise the forces of the last
 * sweep are kept (f = (f_potential + f_interactions) + f_frame).  ret: 0 on convergence, else
 * max_iter + 1 (FQSB_ERR_NO_CONVERGENCE when max_iter_is_error). */
int fqsb_minimise_nopassing(fqsb_system* h, double tol, uint64_t niter_tol, uint64_t max_iter, int max_iter_is_error,
                            uint64_t* ret);
int fqsb_minimise_truncate(fqsb_system* h, const int64_t* i_n, uint64_t A_truncate, uint64_t S_truncate, double tol,
                           uint64_t niter_tol, uint64_t max_iter, int time_activity, int max_iter_is_error,
                           uint64_t* ret);                         /* minimise_truncate main.cpp:172-184, detail.h:1833 */
int fqsb_max_uniform_displacement(fqsb_system* h, int direction, double* ret); /* main.cpp:136-141, detail.h:1901 */
int fqsb_event_driven_step(fqsb_system* h, double eps, int kick, int direction,
                           double* ret);                           /* eventDrivenStep  main.cpp:186-193, detail.h:1933 */
int fqsb_trigger(fqsb_system* h, int64_t p, double eps, int direction); /* trigger     main.cpp:143-150, detail.h:1972 */
int fqsb_advance_to_fixed_force(fqsb_system* h, double f_frame, int allow_plastic); /* main.cpp:152-158, detail.h:1988 */
int fqsb_quench(fqsb_system* h);                                  /* quench           main.cpp:131, detail.h:1527 */
int fqsb_refresh(fqsb_system* h);                                 /* refresh          main.cpp:130, detail.h:1310 */

/* State transfer (host buffers of size N, C order). */
int fqsb_get_field(fqsb_system* h, int field, double* out);       /* u/v/a/f/f_* getters main.cpp:80-127 */
int fqsb_set_field(fqsb_system* h, int field, const double* in);  /* u/v/a setters main.cpp:80-99, detail.h:1231-1259 */
int fqsb_get_scalar(fqsb_system* h, int which, double* out);
int fqsb_set_u_frame(fqsb_system* h, double u_frame);             /* u_frame setter main.cpp:104, detail.h:1253 */
int fqsb_get_inc(fqsb_system* h, int64_t* inc);                   /* inc getter main.cpp:102 */
int fqsb_set_inc(fqsb_system* h, int64_t inc);                    /* inc setter main.cpp:102, detail.h:1212 */
int fqsb_set_t(fqsb_system* h, double t);                         /* t setter main.cpp:103, detail.h:1200 */
int fqsb_quasistatic_activity(fqsb_system* h, int64_t* first, int64_t* last); /* main.cpp:195-201, detail.h:1802-1818 */

/* Chunk (prrng pcg32_tensor_cumsum members used through system.chunk, tests/test_Line1d.py:83-86,309-341). */
int fqsb_get_index(fqsb_system* h, int64_t* index_at_align, int64_t* chunk_index_at_align, double* left_of_align,
                   double* right_of_align);                        /* any pointer may be NULL */
int fqsb_chunk_size(fqsb_system* h, int64_t* nchunk);
int fqsb_chunk_data(fqsb_system* h, double* data, int64_t* start); /* data [N, nchunk]; either may be NULL */
int fqsb_chunk_state_at(fqsb_system* h, const int64_t* index, uint64_t* state);
int fqsb_chunk_restore(fqsb_system* h, const uint64_t* state, const double* value, const int64_t* index);

/*
 * RandomNormalForcing (thermal forcing): Line1d.System_Cuspy_Laplace_RandomForcing (Line1d.h:264-330,
 * main.cpp:570-621), Line1d.System_Cuspy_Quartic_RandomForcing (main.cpp:623-676) and
 * Particles.System_Cuspy_RandomForcing (main.cpp:335-384); the force itself is
 * detail::RandomNormalForcing, detail.h:881-1000.  Every time step (inc++ first), each particle with
 * inc >= next[p] redraws f_thermal[p] = mean + (stddev sqrt 2) erfinv(2 r - 1), r = u32 2^-32, from one
 * pcg32 stream (seeded with `seed` on the default PCG stream), in particle order, and next[p] +=
 * dinc[p]; f = ((((f_frame + f_potential) + f_interactions) + f_damping) + f_thermal).  Attach once,
 * right after fqsb_create (the reference constructs it with the system): it draws at the current inc
 * as the constructor's refresh does.  Cuspy potential with Laplace1d, Quartic1d or no interactions.
 * fqsb_set_inc and fqsb_refresh draw as updated_inc does (detail.h:1241-1247, 1310-1315, 1369-1375).
 */
int fqsb_set_random_forcing(fqsb_system* h, double mean, double stddev, uint64_t seed, const int64_t* dinc_init,
                            const int64_t* dinc);
/* system.external members (main.cpp:253-269): the stream's state, f_thermal [N] and next [N]; any
 * pointer may be NULL.  Setting f_thermal leaves f as it is until the next force update, as
 * RandomNormalForcing::set_f_thermal does. */
int fqsb_random_forcing_get(fqsb_system* h, uint64_t* state, double* f_thermal, int64_t* next);
int fqsb_random_forcing_set(fqsb_system* h, const uint64_t* state, const double* f_thermal, const int64_t* next);

/*
 * Device-resident variants for callers that keep data on the GPU (pointers
 * are device pointers of N doubles on the handle's device).
 */
int fqsb_get_field_device(fqsb_system* h, int field, double* out_device);
int fqsb_set_field_device(fqsb_system* h, int field, const double* in_device);

/* Timing support: the stream the handle launches on (a cudaStream_t). */
int fqsb_get_stream(fqsb_system* h, void** stream);

/*
 * Parameters mu, k_interactions and eta of an existing system (no counterpart in the reference, whose
 * parameters are fixed at construction; needed to differentiate with respect to them).
 */
int fqsb_set_parameters(fqsb_system* h, double mu, double k_interactions, double eta);

/*
 * Adjoint of a trajectory (no counterpart in the reference).  From the current state x_0 = (u, v, a),
 * fqsb_adjoint_forward runs T steps with u_frame = schedule[t] set before step t (host array of T),
 * keeps checkpoints every K steps, and returns
 *     loss = (1/last) sum_{t = T-last}^{T-1} mean_p f_frame_t[p] + 0.5 mean_p u_T[p]^2 ;
 * the system is left in x_T.  fqsb_adjoint_backward then recomputes each K-step segment from its
 * checkpoint and runs the hand-written adjoint step backwards, giving dL/du_0, dL/dv_0 (host arrays of
 * N), dL/dschedule (host array of T) and grad_params = {dL/dmu, dL/dk_interactions, dL/deta}.
 * Exact for Smooth and SemiSmooth; for Cuspy the wells are held at the forward's.  Line1d / Particles.
 */
int fqsb_adjoint_forward(fqsb_system* h, const double* schedule, int64_t T, int64_t K, int64_t last, double* loss);
int fqsb_adjoint_backward(fqsb_system* h, double* grad_u0, double* grad_v0, double* grad_schedule, double* grad_params);
/* As fqsb_adjoint_backward, with dL/du_0 and dL/dv_0 written to device arrays of N doubles on the handle's
 * device (for callers whose tensors live on the GPU); grad_schedule and grad_params stay host arrays. */
int fqsb_adjoint_backward_device(fqsb_system* h, double* grad_u0_device, double* grad_v0_device,
                                 double* grad_schedule, double* grad_params);

/*
 * Batched form: many independent Line1d System_Cuspy_Laplace realisations of uneven size (realisation j:
 * sizes[j] particles, pcg32 initstate seeds[j] + p, frame stiffness k_frame[j]; shared m, eta, mu,
 * k_interactions, dt, distribution, offset, nchunk) on one GPU.  No counterpart in the reference,
 * which runs one System at a time; each realisation follows exactly the plain path's arithmetic.
 * `window` (34 <= window <= nchunk) is the number of yield positions kept per particle; the yield
 * sequence does not depend on it.  threads (32..256) x ppt (1 or 2) is the tile (0: defaults, 256 x 2).
 */
typedef struct {
    int64_t n_instances;
    const int64_t* sizes;
    const uint64_t* seeds;
    const double* k_frame;
    double m, eta, mu, k_interactions, dt;
    int distribution;
    int n_parameters;
    double parameters[4];
    double offset;
    int64_t nchunk;
    int64_t window;
    int threads, ppt;
    void* stream;
    int device;
} fqsb_batch_config;

typedef struct fqsb_batch fqsb_batch;

int fqsb_batch_create(const fqsb_batch_config* cfg, fqsb_batch** out);
int fqsb_batch_destroy(fqsb_batch* h);
const char* fqsb_batch_last_error(const fqsb_batch* h);
/*
 * ncycles quasistatic cycles per realisation, in one device-side run: each cycle is
 * eventDrivenStep(eps, kick=false), eventDrivenStep(eps, kick=true), minimise(tol, niter_tol, max_iter)
 * (the protocol of the reference's examples/Line1d_Cuspy_Laplace.py:41-60), every realisation
 * converging on its own.  Per realisation and cycle (arrays [n_instances x ncycles]): u_frame, mean
 * f_frame, the avalanche size S = sum(index_at_align - index at the cycle start) and inc after the
 * cycle; status_out[j] = 0, FQSB_ERR_NAN or FQSB_ERR_NO_CONVERGENCE.
 */
int fqsb_batch_quasistatic(fqsb_batch* h, int64_t ncycles, double eps, double tol, uint64_t niter_tol,
                           uint64_t max_iter, double* u_frame_out, double* f_frame_out, int64_t* S_out,
                           int64_t* inc_out, int32_t* status_out);
int fqsb_batch_get(fqsb_batch* h, int64_t instance, int field, double* out); /* u, v or a of one realisation */
int fqsb_batch_get_index(fqsb_batch* h, int64_t instance, int64_t* index_at_align);
int fqsb_batch_frame(fqsb_batch* h, double* u_frame); /* u_frame of every realisation */

/*
 * Residual |f| / |f_frame| (|f| when |f_frame| == 0) of two device arrays of n doubles, in the same
 * fixed pairwise summation order as FQSB_SCALAR_RESIDUAL, written to the device double
 * *residual_device; enqueued on `stream` (a cudaStream_t, NULL = default stream) and asynchronous,
 * unlike the other entry points.  No counterpart in the reference: it exists for callers that cannot
 * allocate device memory (inside a global-mode stream capture, under another framework's memory
 * pool, or in loops that cannot afford cudaFree's implicit synchronisation).  It allocates nothing:
 * its scratch is a fixed 512 KiB device array shared by all calls, so n <= FQSB_NOALLOC_MAX_N
 * (larger n fails with FQSB_ERR_INVALID) and calls that overlap on the GPU race.  The first call on a
 * device looks up the scratch address; make it before any stream capture begins.
 */
#define FQSB_NOALLOC_MAX_N ((int64_t)1 << 25)
int fqsb_residual_noalloc(const double* f_device, const double* f_frame_device, int64_t n, double* residual_device,
                          void* stream);

/*
 * Measurement support (no counterpart in the reference): binary64 operations per second of this GPU for
 * op = 0 (add), 1 (mul) or 2 (fma), with n_soft of 8 independent chains per thread in the integer-pipe
 * form the step kernels use (0 = all on the fp64 pipe; fma: 0 only).  The fp64 roofline denominator of
 * the step kernel.  Allocates and frees a small output buffer; runs two launches of ~10 ms.
 */
int fqsb_measure_arith(int device, int op, int n_soft, double* gops);

/* Build information: "fqsb <version> sm_103a". */
const char* fqsb_version(void);

#ifdef __cplusplus
}
#endif

#endif
