/*
 * fqsb.hpp -- header-only C++ classes over the C ABI of include/fqsb.h.
 *
 * They mirror the reference's C++ API (include/FrictionQPotSpringBlock/Line1d.h, Line2d.h,
 * Particles.h and the System methods of detail.h) for the time-integration path: same class names,
 * constructor arguments and defaults, method names; errors throw std::runtime_error with the
 * reference's messages.  State accessors return std::vector copies (the reference returns views).
 */
#ifndef FQSB_HPP
#define FQSB_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "fqsb.h"

namespace FrictionQPotSpringBlock_gb300 {

inline int distribution_id(const std::string& name)
{
    /* string_to_distribution, detail.h:31-66 */
    if (name == "random") return FQSB_DIST_RANDOM;
    if (name == "delta") return FQSB_DIST_DELTA;
    if (name == "exponential") return FQSB_DIST_EXPONENTIAL;
    if (name == "power") return FQSB_DIST_POWER;
    if (name == "gamma") return FQSB_DIST_GAMMA;
    if (name == "pareto") return FQSB_DIST_PARETO;
    if (name == "weibull") return FQSB_DIST_WEIBULL;
    if (name == "normal") return FQSB_DIST_NORMAL;
    throw std::runtime_error("Unknown distribution: " + name);
}

/* system.external() of the RandomForcing systems (detail::RandomNormalForcing, detail.h:881-1000):
 * the pcg32 state of the draws, the thermal forces and each particle's next draw increment. */
class RandomNormalForcing {
    fqsb_system* m_h = nullptr;
    int64_t m_N = 0;

    void check(int status) const
    {
        if (status != FQSB_OK) {
            throw std::runtime_error(fqsb_last_error(m_h));
        }
    }

public:
    void bind(fqsb_system* h, int64_t N)
    {
        m_h = h;
        m_N = N;
    }
    uint64_t state() const
    {
        uint64_t s = 0;
        check(fqsb_random_forcing_get(m_h, &s, nullptr, nullptr));
        return s;
    }
    void set_state(uint64_t s) { check(fqsb_random_forcing_set(m_h, &s, nullptr, nullptr)); }
    std::vector<double> f_thermal() const
    {
        std::vector<double> out((size_t)m_N);
        check(fqsb_random_forcing_get(m_h, nullptr, out.data(), nullptr));
        return out;
    }
    void set_f_thermal(const std::vector<double>& f)
    {
        if ((int64_t)f.size() != m_N) {
            throw std::runtime_error("assertion failed (xt::has_shape(f_thermal, m_f_thermal.shape()))");
        }
        check(fqsb_random_forcing_set(m_h, nullptr, f.data(), nullptr));
    }
    std::vector<ptrdiff_t> next() const
    {
        std::vector<int64_t> out((size_t)m_N);
        check(fqsb_random_forcing_get(m_h, nullptr, nullptr, out.data()));
        return std::vector<ptrdiff_t>(out.begin(), out.end());
    }
    void set_next(const std::vector<ptrdiff_t>& n)
    {
        if ((int64_t)n.size() != m_N) {
            throw std::runtime_error("assertion failed (xt::has_shape(next, m_next.shape()))");
        }
        std::vector<int64_t> v(n.begin(), n.end());
        check(fqsb_random_forcing_set(m_h, nullptr, nullptr, v.data()));
    }
};

/* Generic system (detail::System, detail.h:1046-2051) resident on one GPU. */
class System {
protected:
    fqsb_system* m_h = nullptr;
    int64_t m_N = 0;
    double m_dt = 0, m_mu = 0, m_eta = 0, m_m = 0, m_k_frame = 0;

    void check(int status) const
    {
        if (status != FQSB_OK) {
            throw std::runtime_error(fqsb_last_error(m_h));
        }
    }

    void init(int potential, int interactions, int64_t rows, int64_t cols, double m, double eta, double mu,
              double kappa, double k_interactions, double k_frame, double dt, uint64_t seed,
              const std::string& distribution, const std::vector<double>& parameters, double offset, size_t nchunk,
              double ip0 = 0.0, double ip1 = 0.0)
    {
        if (parameters.size() > 4) {
            throw std::runtime_error("at most 4 distribution parameters");
        }
        fqsb_config c = {};
        c.potential = potential;
        c.interactions = interactions;
        c.rows = rows;
        c.cols = cols;
        c.m = m;
        c.eta = eta;
        c.mu = mu;
        c.kappa = kappa;
        c.k_interactions = k_interactions;
        c.k_frame = k_frame;
        c.dt = dt;
        c.seed = seed;
        c.distribution = distribution_id(distribution);
        c.n_parameters = (int)parameters.size();
        for (size_t i = 0; i < parameters.size(); ++i) {
            c.parameters[i] = parameters[i];
        }
        c.offset = offset;
        c.offset_per_particle = nullptr;
        c.nchunk = (int64_t)nchunk;
        c.stream = nullptr;
        c.device = 0;
        c.interaction_parameters[0] = ip0;
        c.interaction_parameters[1] = ip1;
        if (fqsb_create(&c, &m_h) != FQSB_OK) {
            throw std::runtime_error(fqsb_last_error(nullptr));
        }
        m_N = rows * cols;
        m_dt = dt;
        m_mu = mu;
        m_eta = eta;
        m_m = m;
        m_k_frame = k_frame;
    }

    RandomNormalForcing m_ext;

    /* RandomNormalForcing constructor (detail.h:903-919) + the system constructor's refresh */
    void attach_random_forcing(double mean, double stddev, uint64_t seed_forcing,
                               const std::vector<ptrdiff_t>& dinc_init, const std::vector<ptrdiff_t>& dinc)
    {
        if ((int64_t)dinc_init.size() != m_N || (int64_t)dinc.size() != m_N) {
            throw std::runtime_error("dinc_init and dinc must have one entry per particle");
        }
        std::vector<int64_t> a(dinc_init.begin(), dinc_init.end()), b(dinc.begin(), dinc.end());
        check(fqsb_set_random_forcing(m_h, mean, stddev, seed_forcing, a.data(), b.data()));
        m_ext.bind(m_h, m_N);
    }

    std::vector<double> field(int which) const
    {
        std::vector<double> out((size_t)m_N);
        check(fqsb_get_field(m_h, which, out.data()));
        return out;
    }

    double scalar(int which) const
    {
        double out = 0;
        check(fqsb_get_scalar(m_h, which, &out));
        return out;
    }

public:
    System() = default;
    System(const System&) = delete;
    System& operator=(const System&) = delete;
    virtual ~System()
    {
        if (m_h) {
            fqsb_destroy(m_h);
        }
    }

    size_t size() const { return (size_t)m_N; }
    double dt() const { return m_dt; }
    double mu() const { return m_mu; }
    double eta() const { return m_eta; }
    double m() const { return m_m; }
    double k_frame() const { return m_k_frame; }

    std::vector<double> u() const { return field(FQSB_FIELD_U); }
    std::vector<double> v() const { return field(FQSB_FIELD_V); }
    std::vector<double> a() const { return field(FQSB_FIELD_A); }
    std::vector<double> f() const { return field(FQSB_FIELD_F); }
    std::vector<double> f_potential() const { return field(FQSB_FIELD_F_POTENTIAL); }
    std::vector<double> f_interactions() const { return field(FQSB_FIELD_F_INTERACTIONS); }
    std::vector<double> f_frame() const { return field(FQSB_FIELD_F_FRAME); }
    std::vector<double> f_damping() const { return field(FQSB_FIELD_F_DAMPING); }

    void set_u(const std::vector<double>& x) { check(fqsb_set_field(m_h, FQSB_FIELD_U, x.data())); }
    void set_v(const std::vector<double>& x) { check(fqsb_set_field(m_h, FQSB_FIELD_V, x.data())); }
    void set_a(const std::vector<double>& x) { check(fqsb_set_field(m_h, FQSB_FIELD_A, x.data())); }

    double u_frame() const { return scalar(FQSB_SCALAR_U_FRAME); }
    void set_u_frame(double x) { check(fqsb_set_u_frame(m_h, x)); }
    double t() const { return scalar(FQSB_SCALAR_T); }
    void set_t(double x) { check(fqsb_set_t(m_h, x)); }
    int64_t inc() const
    {
        int64_t i = 0;
        check(fqsb_get_inc(m_h, &i));
        return i;
    }
    void set_inc(int64_t i) { check(fqsb_set_inc(m_h, i)); }
    double temperature() const { return scalar(FQSB_SCALAR_TEMPERATURE); }
    double residual() const { return scalar(FQSB_SCALAR_RESIDUAL); }

    std::vector<int64_t> index_at_align() const
    {
        std::vector<int64_t> out((size_t)m_N);
        check(fqsb_get_index(m_h, out.data(), nullptr, nullptr, nullptr));
        return out;
    }

    void refresh() { check(fqsb_refresh(m_h)); }
    void quench() { check(fqsb_quench(m_h)); }
    void timeStep() { check(fqsb_time_step(m_h)); }
    void timeSteps(size_t n) { check(fqsb_time_steps(m_h, n)); }
    void flowSteps(size_t n, double v_frame) { check(fqsb_flow_steps(m_h, n, v_frame)); }

    size_t timeStepsUntilEvent(double tol = 1e-5, size_t niter_tol = 10, size_t max_iter = 1e9)
    {
        uint64_t r = 0;
        check(fqsb_time_steps_until_event(m_h, tol, niter_tol, max_iter, &r));
        return (size_t)r;
    }

    size_t minimise(double tol = 1e-5, size_t niter_tol = 10, size_t max_iter = 1e9, bool time_activity = false,
                    bool max_iter_is_error = true)
    {
        uint64_t r = 0;
        check(fqsb_minimise(m_h, tol, niter_tol, max_iter, time_activity, max_iter_is_error, &r));
        return (size_t)r;
    }

    size_t minimise_truncate(const std::vector<int64_t>& i_n, size_t A_truncate = 0, size_t S_truncate = 0,
                             double tol = 1e-5, size_t niter_tol = 10, size_t max_iter = 1e9,
                             bool time_activity = true, bool max_iter_is_error = true)
    {
        uint64_t r = 0;
        check(fqsb_minimise_truncate(m_h, i_n.data(), A_truncate, S_truncate, tol, niter_tol, max_iter, time_activity,
                                     max_iter_is_error, &r));
        return (size_t)r;
    }

    double maxUniformDisplacement(int direction = 1)
    {
        double r = 0;
        check(fqsb_max_uniform_displacement(m_h, direction, &r));
        return r;
    }

    double eventDrivenStep(double eps, bool kick, int direction = 1)
    {
        double r = 0;
        check(fqsb_event_driven_step(m_h, eps, kick, direction, &r));
        return r;
    }

    void trigger(size_t p, double eps, int direction = 1) { check(fqsb_trigger(m_h, (int64_t)p, eps, direction)); }
    void advanceToFixedForce(double f_frame, bool allow_plastic = false)
    {
        check(fqsb_advance_to_fixed_force(m_h, f_frame, allow_plastic));
    }

    size_t quasistaticActivityFirst() const
    {
        int64_t a = 0, b = 0;
        check(fqsb_quasistatic_activity(m_h, &a, &b));
        return (size_t)a;
    }
    size_t quasistaticActivityLast() const
    {
        int64_t a = 0, b = 0;
        check(fqsb_quasistatic_activity(m_h, &a, &b));
        return (size_t)b;
    }
};

namespace Line1d {

/* Line1d.h:112-162 */
class System_Cuspy_Laplace : public System {
public:
    System_Cuspy_Laplace(double m, double eta, double mu, double k_interactions, double k_frame, double dt,
                         const std::array<size_t, 1>& shape, uint64_t seed, const std::string& distribution,
                         const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_LAPLACE1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, k_interactions, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }
};

/* Line1d.h:336-377 */
class System_SemiSmooth_Laplace : public System {
public:
    System_SemiSmooth_Laplace(double m, double eta, double mu, double kappa, double k_interactions, double k_frame,
                              double dt, const std::array<size_t, 1>& shape, uint64_t seed,
                              const std::string& distribution, const std::vector<double>& parameters,
                              double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_SEMISMOOTH, FQSB_LAPLACE1D, 1, (int64_t)shape[0], m, eta, mu, kappa, k_interactions, k_frame, dt,
             seed, distribution, parameters, offset, nchunk);
    }
};

/* Line1d.h:379-422 */
class System_Smooth_Laplace : public System {
public:
    System_Smooth_Laplace(double m, double eta, double mu, double k_interactions, double k_frame, double dt,
                          const std::array<size_t, 1>& shape, uint64_t seed, const std::string& distribution,
                          const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_SMOOTH, FQSB_LAPLACE1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, k_interactions, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }
};

/* Line1d.h:173-238: Cuspy + Laplace1d minimised with the no-passing rule (m = 1, no dynamics) */
class System_Cuspy_Laplace_Nopassing : public System {
public:
    System_Cuspy_Laplace_Nopassing(double mu, double k_interactions, double k_frame, const std::array<size_t, 1>& shape,
                                   uint64_t seed, const std::string& distribution,
                                   const std::vector<double>& parameters, double offset = -100.0,
                                   size_t nchunk = 5000, double eta = 0.0, double dt = 0.0)
    {
        init(FQSB_CUSPY, FQSB_LAPLACE1D, 1, (int64_t)shape[0], 1.0, eta, mu, 0.0, k_interactions, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }

    /* detail.h:1694-1753 */
    size_t minimise(double tol = 1e-5, size_t niter_tol = 10, size_t max_iter = 1e9, bool time_activity = false,
                    bool max_iter_is_error = true)
    {
        if (time_activity) {
            throw std::runtime_error("assertion failed (!time_activity)");
        }
        uint64_t r = 0;
        check(fqsb_minimise_nopassing(m_h, tol, niter_tol, max_iter, max_iter_is_error, &r));
        return (size_t)r;
    }
};

/* Line1d.h:264-330: Cuspy + Laplace1d with RandomNormalForcing */
class System_Cuspy_Laplace_RandomForcing : public System {
public:
    System_Cuspy_Laplace_RandomForcing(double m, double eta, double mu, double k_interactions, double k_frame,
                                       double dt, double mean, double stddev, uint64_t seed_forcing,
                                       const std::vector<ptrdiff_t>& dinc_init, const std::vector<ptrdiff_t>& dinc,
                                       const std::array<size_t, 1>& shape, uint64_t seed,
                                       const std::string& distribution, const std::vector<double>& parameters,
                                       double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_LAPLACE1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, k_interactions, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
        attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc);
    }
    RandomNormalForcing* external() { return &m_ext; }
};

/* Line1d.h:486-556: Cuspy + Quartic1d with RandomNormalForcing */
class System_Cuspy_Quartic_RandomForcing : public System {
public:
    System_Cuspy_Quartic_RandomForcing(double m, double eta, double mu, double a1, double a2, double k_frame,
                                       double dt, double mean, double stddev, uint64_t seed_forcing,
                                       const std::vector<ptrdiff_t>& dinc_init, const std::vector<ptrdiff_t>& dinc,
                                       const std::array<size_t, 1>& shape, uint64_t seed,
                                       const std::string& distribution, const std::vector<double>& parameters,
                                       double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_QUARTIC1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed, distribution,
             parameters, offset, nchunk, a1, a2);
        attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc);
    }
    RandomNormalForcing* external() { return &m_ext; }
};

/* Line1d.h:428-481 */
class System_Cuspy_Quartic : public System {
public:
    System_Cuspy_Quartic(double m, double eta, double mu, double a1, double a2, double k_frame, double dt,
                         const std::array<size_t, 1>& shape, uint64_t seed, const std::string& distribution,
                         const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_QUARTIC1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed, distribution,
             parameters, offset, nchunk, a1, a2);
    }
};

/* Line1d.h:562-615 */
class System_Cuspy_QuarticGradient : public System {
public:
    System_Cuspy_QuarticGradient(double m, double eta, double mu, double k2, double k4, double k_frame, double dt,
                                 const std::array<size_t, 1>& shape, uint64_t seed, const std::string& distribution,
                                 const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_QUARTICGRADIENT1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed,
             distribution, parameters, offset, nchunk, k2, k4);
    }
};

/* Line1d.h:617-675 */
class System_Cuspy_LongRange : public System {
public:
    System_Cuspy_LongRange(double m, double eta, double mu, double k_interactions, double alpha, double k_frame,
                           double dt, const std::array<size_t, 1>& shape, uint64_t seed,
                           const std::string& distribution, const std::vector<double>& parameters,
                           double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_LONGRANGE1D, 1, (int64_t)shape[0], m, eta, mu, 0.0, k_interactions, k_frame, dt, seed,
             distribution, parameters, offset, nchunk, alpha, 0.0);
    }
};

} // namespace Line1d

namespace Line2d {

/* Line2d.h:77-116 */
class System_Cuspy_Laplace : public System {
public:
    System_Cuspy_Laplace(double m, double eta, double mu, double k_interactions, double k_frame, double dt,
                         const std::array<size_t, 2>& shape, uint64_t seed, const std::string& distribution,
                         const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_LAPLACE2D, (int64_t)shape[0], (int64_t)shape[1], m, eta, mu, 0.0, k_interactions,
             k_frame, dt, seed, distribution, parameters, offset, nchunk);
    }
};

/* Line2d.h:122-167 */
class System_Cuspy_QuarticGradient : public System {
public:
    System_Cuspy_QuarticGradient(double m, double eta, double mu, double k2, double k4, double k_frame, double dt,
                                 const std::array<size_t, 2>& shape, uint64_t seed, const std::string& distribution,
                                 const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_QUARTICGRADIENT2D, (int64_t)shape[0], (int64_t)shape[1], m, eta, mu, 0.0, 0.0, k_frame,
             dt, seed, distribution, parameters, offset, nchunk, k2, k4);
    }
};

} // namespace Line2d

namespace Particles {

/* Particles.h:93-311 (no interactions) */
class System_Cuspy : public System {
public:
    System_Cuspy(double m, double eta, double mu, double k_frame, double dt, const std::array<size_t, 1>& shape,
                 uint64_t seed, const std::string& distribution, const std::vector<double>& parameters,
                 double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_INTERACTIONS_NONE, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }
};

/* Particles.h:161-227: independent Cuspy particles with RandomNormalForcing */
class System_Cuspy_RandomForcing : public System {
public:
    System_Cuspy_RandomForcing(double m, double eta, double mu, double k_frame, double dt, double mean, double stddev,
                               uint64_t seed_forcing, const std::vector<ptrdiff_t>& dinc_init,
                               const std::vector<ptrdiff_t>& dinc, const std::array<size_t, 1>& shape, uint64_t seed,
                               const std::string& distribution, const std::vector<double>& parameters,
                               double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_CUSPY, FQSB_INTERACTIONS_NONE, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
        attach_random_forcing(mean, stddev, seed_forcing, dinc_init, dinc);
    }
    RandomNormalForcing* external() { return &m_ext; }
};

class System_SemiSmooth : public System {
public:
    System_SemiSmooth(double m, double eta, double mu, double kappa, double k_frame, double dt,
                      const std::array<size_t, 1>& shape, uint64_t seed, const std::string& distribution,
                      const std::vector<double>& parameters, double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_SEMISMOOTH, FQSB_INTERACTIONS_NONE, 1, (int64_t)shape[0], m, eta, mu, kappa, 0.0, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }
};

class System_Smooth : public System {
public:
    System_Smooth(double m, double eta, double mu, double k_frame, double dt, const std::array<size_t, 1>& shape,
                  uint64_t seed, const std::string& distribution, const std::vector<double>& parameters,
                  double offset = -100.0, size_t nchunk = 5000)
    {
        init(FQSB_SMOOTH, FQSB_INTERACTIONS_NONE, 1, (int64_t)shape[0], m, eta, mu, 0.0, 0.0, k_frame, dt, seed,
             distribution, parameters, offset, nchunk);
    }
};

} // namespace Particles

} // namespace FrictionQPotSpringBlock_gb300

#endif
