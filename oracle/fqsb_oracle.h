/*
 * CPU oracle for the FrictionQPotSpringBlock time-integration path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * arithmetic, used by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline as the checker.  The product (frictionqpotspringblock_gb300) never
 * links, imports or calls it.
 *
 * Reference followed (paths inside the reference project):
 *   include/FrictionQPotSpringBlock/detail.h   System, Cuspy, SemiSmooth, Smooth,
 *                                              Laplace1d, Laplace2d
 *   include/FrictionQPotSpringBlock/Line1d.h   seeding (initstate = seed + p,
 *   include/FrictionQPotSpringBlock/Line2d.h   initseq = 0), global offset
 *   prrng (third-party, not in the reference tree; pcg32 + cumsum chunk)
 *   GooseFEM::Iterate::StopList (third-party; residual window)
 *
 * Parity pinning: the pcg32 stream, the "random" and "delta" transforms, the
 * cumulative-sum chunk with forward regeneration and the dynamics are pinned
 * by the reference's historic golden trajectories (examples directory, .h5 files) and by its
 * analytic unit tests; see tests/test_oracle_golden.py.
 */
#ifndef FQSB_ORACLE_H
#define FQSB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oq_system oq_system;

/* potential */
#define OQ_CUSPY 0
#define OQ_SEMISMOOTH 1
#define OQ_SMOOTH 2
/* interactions */
#define OQ_NONE 0
#define OQ_LAPLACE1D 1
#define OQ_LAPLACE2D 2
#define OQ_QUARTIC1D 3
#define OQ_QUARTICGRAD1D 4
#define OQ_QUARTICGRAD2D 5
#define OQ_LONGRANGE1D 6
/* distributions (prrng names) */
#define OQ_DIST_RANDOM 0
#define OQ_DIST_DELTA 1
#define OQ_DIST_EXPONENTIAL 2
#define OQ_DIST_POWER 3
#define OQ_DIST_GAMMA 4
#define OQ_DIST_PARETO 5
#define OQ_DIST_WEIBULL 6
#define OQ_DIST_NORMAL 7
/* reduction order of norms / sums */
#define OQ_SUM_SEQUENTIAL 0 /* the reference's loop order */
#define OQ_SUM_PAIRWISE 1   /* fixed pairwise tree over the flat index (the device's order) */
/* elementary functions used by transforms and the Smooth potential */
#define OQ_MATH_LIBM 0     /* host libm, as the reference */
#define OQ_MATH_PORTABLE 1 /* the product's deterministic fq_math.h */

/* status codes (mirror the C-ABI) */
#define OQ_OK 0
#define OQ_ERR_NAN 1
#define OQ_ERR_NO_CONVERGENCE 2
#define OQ_ERR_INVALID 3
#define OQ_ERR_NOT_POSSIBLE 6
#define OQ_ERR_REQUIRE 7
#define OQ_ERR_UNSUPPORTED 8

oq_system* oq_create(
    int potential, int interactions, int64_t rows, int64_t cols,
    double m, double eta, double mu, double kappa, double k_interactions, double k_frame, double dt,
    uint64_t seed, int distribution, const double* parameters, int n_parameters,
    double offset, const double* offset_per_particle, int64_t nchunk,
    int sum_mode, int math_mode);
void oq_destroy(oq_system* s);
const char* oq_last_error(oq_system* s);
int64_t oq_size(oq_system* s);

/* raw pcg32 / transform probes */
uint32_t oq_pcg32_stream(uint64_t initstate, uint64_t initseq, int64_t n, uint32_t* out);
uint64_t oq_pcg32_advance(uint64_t state, uint64_t inc, int64_t delta);
double oq_transform(int distribution, const double* parameters, int n_parameters, uint32_t r, int math_mode);
double oq_math(int which, double x, double y, int math_mode);

/* state access */
int oq_get(oq_system* s, int field, double* out);
int oq_set(oq_system* s, int field, const double* in);
double oq_get_scalar(oq_system* s, int which);
int oq_set_u_frame(oq_system* s, double v);
int oq_set_inc(oq_system* s, int64_t inc);
int64_t oq_get_inc(oq_system* s);
int oq_set_t(oq_system* s, double t);
int oq_get_index(oq_system* s, int64_t* gidx, int64_t* cidx, double* left, double* right);
int oq_chunk_data(oq_system* s, double* out, int64_t* start);
int oq_chunk_state_at(oq_system* s, const int64_t* index, uint64_t* state);
int oq_chunk_restore(oq_system* s, const uint64_t* state, const double* value, const int64_t* index);
int oq_yield_sequence(oq_system* s, int64_t p, int64_t k0, int64_t count, double* out);
int oq_sequence(uint64_t seed, int64_t p, int distribution, const double* parameters, int n_parameters, double offset,
                int64_t nchunk, int math_mode, int64_t k0, int64_t count, double* out);
int64_t oq_quasistatic_first(oq_system* s);
int64_t oq_quasistatic_last(oq_system* s);

/* dynamics (names follow detail.h) */
int oq_refresh(oq_system* s);
int oq_quench(oq_system* s);
int oq_time_step(oq_system* s);
int oq_time_steps(oq_system* s, uint64_t n);
int oq_flow_steps(oq_system* s, uint64_t n, double v_frame);
int oq_time_steps_until_event(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, uint64_t* ret);
/* System_Cuspy_Laplace_Nopassing::minimise (detail.h:1694-1753) */
int oq_minimise_nopassing(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, int max_iter_is_error,
                          uint64_t* ret);
int oq_set_interaction_parameters(oq_system* s, double a, double b);
int oq_set_thermal(oq_system* s, double mean, double stddev, uint64_t state, uint64_t inc, const int64_t* next,
                   const int64_t* dinc, int mode);
int oq_get_thermal(oq_system* s, double* f_thermal);
/* RandomNormalForcing members state / f_thermal / next (detail.h:947-995); NULL pointers are skipped.
 * Setting f_thermal does not recompute f (set_f_thermal). */
int oq_thermal_get(oq_system* s, uint64_t* state, double* f_thermal, int64_t* next);
int oq_thermal_set(oq_system* s, const uint64_t* state, const double* f_thermal, const int64_t* next);
int oq_minimise(oq_system* s, double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                int max_iter_is_error, uint64_t* ret);
int oq_minimise_truncate(oq_system* s, const int64_t* i_n, uint64_t A_truncate, uint64_t S_truncate,
                         double tol, uint64_t niter_tol, uint64_t max_iter, int time_activity,
                         int max_iter_is_error, uint64_t* ret);
int oq_max_uniform_displacement(oq_system* s, int direction, double* ret);
int oq_event_driven_step(oq_system* s, double eps, int kick, int direction, double* ret);
int oq_trigger(oq_system* s, int64_t p, double eps, int direction);
int oq_advance_to_fixed_force(oq_system* s, double f_frame, int allow_plastic);

/* fields for oq_get / oq_set */
#define OQ_F_U 0
#define OQ_F_V 1
#define OQ_F_A 2
#define OQ_F_F 3
#define OQ_F_F_POTENTIAL 4
#define OQ_F_F_INTERACTIONS 5
#define OQ_F_F_FRAME 6
#define OQ_F_F_DAMPING 7
/* scalars */
#define OQ_S_U_FRAME 0
#define OQ_S_T 1
#define OQ_S_TEMPERATURE 2
#define OQ_S_RESIDUAL 3
#define OQ_S_MEAN_F_FRAME 4

#ifdef __cplusplus
}
#endif

#endif
