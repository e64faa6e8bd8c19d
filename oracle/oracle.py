"""ctypes wrapper of the CPU oracle (fqsb_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline / reference arm, always as the checker.  The product
package never imports this module.

The wrapper classes mirror the reference's Python API
(python/main.cpp:46-226 in the reference project) so that oracle-backed tests
read like the reference's own tests.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libfqsb_oracle.so"
LIB_MT = BUILD / "libfqsb_oracle_mt.so"  # OpenMP build: per-particle loops over the host cores
SOURCES = [HERE / "fqsb_oracle.c", HERE / "fqsb_oracle.h", HERE.parent / "frictionqpotspringblock_gb300" / "csrc" / "fq_math.h"]

CUSPY, SEMISMOOTH, SMOOTH = 0, 1, 2
NONE, LAPLACE1D, LAPLACE2D, QUARTIC1D, QUARTICGRAD1D, QUARTICGRAD2D, LONGRANGE1D = 0, 1, 2, 3, 4, 5, 6
SUM_SEQUENTIAL, SUM_PAIRWISE = 0, 1
MATH_LIBM, MATH_PORTABLE = 0, 1
DISTRIBUTIONS = {
    "random": 0,
    "delta": 1,
    "exponential": 2,
    "power": 3,
    "gamma": 4,
    "pareto": 5,
    "weibull": 6,
    "normal": 7,
}
F_U, F_V, F_A, F_F, F_POT, F_INT, F_FRAME, F_DAMP = range(8)
S_U_FRAME, S_T, S_TEMPERATURE, S_RESIDUAL, S_MEAN_F_FRAME = range(5)


def build(force: bool = False, threads: bool = False) -> pathlib.Path:
    """Compile the oracle with gcc (no FMA contraction, no fast-math); threads=True builds the OpenMP
    variant, whose per-particle loops run over the host cores with bit-identical results."""
    BUILD.mkdir(exist_ok=True)
    target = LIB_MT if threads else LIB
    newest = max(p.stat().st_mtime for p in SOURCES)
    if force or not target.exists() or target.stat().st_mtime < newest:
        tmp = BUILD / f"{target.stem}.{os.getpid()}.so"
        cmd = [
            "gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            *(["-fopenmp"] if threads else []), "-o", str(tmp), str(HERE / "fqsb_oracle.c"), "-lm",
        ]
        subprocess.run(cmd, check=True)
        os.replace(tmp, target)
    return target


_libs = {}


def lib(threads: bool = False):
    if threads not in _libs:
        L = ctypes.CDLL(str(build(threads=threads)))
        P = ctypes.c_void_p
        d, i64, u64, i32 = ctypes.c_double, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int
        pd = ctypes.POINTER(ctypes.c_double)
        L.oq_create.restype = P
        L.oq_create.argtypes = [i32, i32, i64, i64, d, d, d, d, d, d, d, u64, i32, pd, i32, d, pd, i64, i32, i32]
        L.oq_destroy.argtypes = [P]
        L.oq_last_error.restype = ctypes.c_char_p
        L.oq_last_error.argtypes = [P]
        L.oq_size.restype = i64
        L.oq_size.argtypes = [P]
        L.oq_pcg32_stream.restype = ctypes.c_uint32
        L.oq_pcg32_stream.argtypes = [u64, u64, i64, P]
        L.oq_pcg32_advance.restype = u64
        L.oq_pcg32_advance.argtypes = [u64, u64, i64]
        L.oq_transform.restype = d
        L.oq_transform.argtypes = [i32, pd, i32, ctypes.c_uint32, i32]
        L.oq_math.restype = d
        L.oq_math.argtypes = [i32, d, d, i32]
        L.oq_get.argtypes = [P, i32, P]
        L.oq_set.argtypes = [P, i32, P]
        L.oq_get_scalar.restype = d
        L.oq_get_scalar.argtypes = [P, i32]
        L.oq_set_u_frame.argtypes = [P, d]
        L.oq_set_inc.argtypes = [P, i64]
        L.oq_get_inc.restype = i64
        L.oq_get_inc.argtypes = [P]
        L.oq_set_t.argtypes = [P, d]
        L.oq_get_index.argtypes = [P, P, P, P, P]
        L.oq_chunk_data.argtypes = [P, P, P]
        L.oq_chunk_state_at.argtypes = [P, P, P]
        L.oq_chunk_restore.argtypes = [P, P, P, P]
        L.oq_yield_sequence.argtypes = [P, i64, i64, i64, P]
        L.oq_sequence.argtypes = [u64, i64, i32, pd, i32, d, i64, i32, i64, i64, P]
        L.oq_quasistatic_first.restype = i64
        L.oq_quasistatic_first.argtypes = [P]
        L.oq_quasistatic_last.restype = i64
        L.oq_quasistatic_last.argtypes = [P]
        for name in ("oq_refresh", "oq_quench", "oq_time_step"):
            getattr(L, name).argtypes = [P]
        L.oq_time_steps.argtypes = [P, u64]
        L.oq_flow_steps.argtypes = [P, u64, d]
        L.oq_time_steps_until_event.argtypes = [P, d, u64, u64, ctypes.POINTER(u64)]
        L.oq_minimise.argtypes = [P, d, u64, u64, i32, i32, ctypes.POINTER(u64)]
        L.oq_minimise_nopassing.argtypes = [P, d, u64, u64, i32, ctypes.POINTER(u64)]
        L.oq_set_interaction_parameters.argtypes = [P, d, d]
        L.oq_set_thermal.argtypes = [P, d, d, u64, u64, P, P, i32]
        L.oq_get_thermal.argtypes = [P, pd]
        L.oq_thermal_get.argtypes = [P, P, P, P]
        L.oq_thermal_set.argtypes = [P, P, P, P]
        L.oq_minimise_truncate.argtypes = [P, P, u64, u64, d, u64, u64, i32, i32, ctypes.POINTER(u64)]
        L.oq_max_uniform_displacement.argtypes = [P, i32, pd]
        L.oq_event_driven_step.argtypes = [P, d, i32, i32, pd]
        L.oq_trigger.argtypes = [P, i64, d, i32]
        L.oq_advance_to_fixed_force.argtypes = [P, d, i32]
        _libs[threads] = L
    return _libs[threads]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def pcg32_stream(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().oq_pcg32_stream(initstate, initseq, n, _ptr(out))
    return out


def pcg32_advance(state: int, inc: int, delta: int) -> int:
    return int(lib().oq_pcg32_advance(state, inc, delta))


def transform(distribution: str, parameters, r32: int, math_mode: int = MATH_PORTABLE) -> float:
    par = (ctypes.c_double * 4)(*list(parameters))
    return lib().oq_transform(DISTRIBUTIONS[distribution], par, len(parameters), r32, math_mode)


def math(which: str, x: float, y: float = 0.0, math_mode: int = MATH_PORTABLE) -> float:
    return lib().oq_math({"log": 0, "pow": 1, "sin": 2, "exp": 3, "cos": 4, "erfinv": 5}[which], x, y, math_mode)


def sequence(seed, p, distribution, parameters, offset, nchunk, k0, count, math_mode=MATH_PORTABLE):
    """Canonical yield positions y_k, k in [k0, k0+count), of particle p of a fresh system."""
    par = (ctypes.c_double * 4)(*list(parameters))
    out = np.empty(count)
    rc = lib().oq_sequence(int(seed), int(p), DISTRIBUTIONS[distribution], par, len(parameters), float(offset),
                           int(nchunk), math_mode, int(k0), int(count), _ptr(out))
    if rc:
        raise OracleError("invalid sequence request")
    return out


class OracleError(RuntimeError):
    pass


class _Chunk:
    """The prrng chunk members the reference's tests use (test_Line1d.py:83-86, 309-326)."""

    def __init__(self, sys):
        self._s = sys

    def _idx(self):
        s = self._s
        g = np.empty(s.size, np.int64)
        c = np.empty(s.size, np.int64)
        left = np.empty(s.size)
        right = np.empty(s.size)
        self._s._L.oq_get_index(s._h, _ptr(g), _ptr(c), _ptr(left), _ptr(right))
        shape = s.shape
        return g.reshape(shape), c.reshape(shape), left.reshape(shape), right.reshape(shape)

    @property
    def index_at_align(self):
        return self._idx()[0]

    @property
    def chunk_index_at_align(self):
        return self._idx()[1]

    @property
    def left_of_align(self):
        return self._idx()[2]

    @property
    def right_of_align(self):
        return self._idx()[3]

    @property
    def data(self):
        s = self._s
        out = np.empty((s.size, s.nchunk))
        self._s._L.oq_chunk_data(s._h, _ptr(out), None)
        return out.reshape(tuple(s.shape) + (s.nchunk,))

    @property
    def start(self):
        s = self._s
        out = np.empty(s.size, np.int64)
        self._s._L.oq_chunk_data(s._h, None, _ptr(out))
        return out.reshape(s.shape)

    def state_at(self, index):
        s = self._s
        idx = np.ascontiguousarray(np.broadcast_to(index, s.shape), dtype=np.int64).ravel()
        out = np.empty(s.size, np.uint64)
        self._s._L.oq_chunk_state_at(s._h, _ptr(idx), _ptr(out))
        return out.reshape(s.shape)

    def restore(self, state, value, index):
        s = self._s
        st = np.ascontiguousarray(state, dtype=np.uint64).ravel()
        val = np.ascontiguousarray(value, dtype=np.float64).ravel()
        idx = np.ascontiguousarray(index, dtype=np.int64).ravel()
        self._s._L.oq_chunk_restore(s._h, _ptr(st), _ptr(val), _ptr(idx))


class System:
    """Oracle system with the reference's attribute and method names."""

    def __init__(self, potential, interactions, shape, m, eta, mu, k_interactions, k_frame, dt, seed,
                 distribution, parameters, offset=-100.0, nchunk=5000, kappa=0.0, offset_per_particle=None,
                 sum_mode=SUM_PAIRWISE, math_mode=MATH_PORTABLE, interaction_parameters=None, threads=False):
        shape = [int(i) for i in shape]
        rows, cols = (1, shape[0]) if len(shape) == 1 else (shape[0], shape[1])
        self.shape = shape
        self.size = rows * cols
        self.nchunk = int(nchunk)
        par = (ctypes.c_double * 4)(*list(parameters))
        offp = None
        if offset_per_particle is not None:
            self._offp = np.ascontiguousarray(offset_per_particle, dtype=np.float64).ravel()
            offp = self._offp.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        self._L = lib(threads)
        h = self._L.oq_create(potential, interactions, rows, cols, m, eta, mu, kappa, k_interactions, k_frame, dt,
                            int(seed), DISTRIBUTIONS[distribution], par, len(parameters), offset, offp, nchunk,
                            sum_mode, math_mode)
        if not h:
            raise OracleError("invalid oracle configuration")
        self._h = h
        if interaction_parameters is not None:
            a, b = (float(x) for x in interaction_parameters)
            self._check(self._L.oq_set_interaction_parameters(h, a, b))
        self.dt, self.mu, self.eta, self.m, self.k_frame = dt, mu, eta, m, k_frame
        self.chunk = _Chunk(self)

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.oq_destroy(self._h)
            self._h = None

    def _check(self, rc):
        if rc != 0:
            raise OracleError(self._L.oq_last_error(self._h).decode())

    def _get(self, field):
        out = np.empty(self.size)
        self._L.oq_get(self._h, field, _ptr(out))
        return out.reshape(self.shape)

    def _set(self, field, value):
        arr = np.ascontiguousarray(np.broadcast_to(value, self.shape), dtype=np.float64)
        self._check(self._L.oq_set(self._h, field, _ptr(arr)))

    u = property(lambda s: s._get(F_U), lambda s, x: s._set(F_U, x))
    v = property(lambda s: s._get(F_V), lambda s, x: s._set(F_V, x))
    a = property(lambda s: s._get(F_A), lambda s, x: s._set(F_A, x))
    f = property(lambda s: s._get(F_F))
    f_potential = property(lambda s: s._get(F_POT))
    f_interactions = property(lambda s: s._get(F_INT))
    f_frame = property(lambda s: s._get(F_FRAME))
    f_damping = property(lambda s: s._get(F_DAMP))
    temperature = property(lambda s: s._L.oq_get_scalar(s._h, S_TEMPERATURE))
    residual = property(lambda s: s._L.oq_get_scalar(s._h, S_RESIDUAL))
    mean_f_frame = property(lambda s: s._L.oq_get_scalar(s._h, S_MEAN_F_FRAME))
    quasistaticActivityFirst = property(lambda s: s._L.oq_quasistatic_first(s._h))
    quasistaticActivityLast = property(lambda s: s._L.oq_quasistatic_last(s._h))

    @property
    def u_frame(self):
        return self._L.oq_get_scalar(self._h, S_U_FRAME)

    @u_frame.setter
    def u_frame(self, value):
        self._L.oq_set_u_frame(self._h, float(value))

    @property
    def inc(self):
        return self._L.oq_get_inc(self._h)

    @inc.setter
    def inc(self, value):
        self._L.oq_set_inc(self._h, int(value))

    @property
    def t(self):
        return self._L.oq_get_scalar(self._h, S_T)

    @t.setter
    def t(self, value):
        self._L.oq_set_t(self._h, float(value))

    @property
    def i(self):
        return self.chunk.index_at_align

    def refresh(self):
        self._L.oq_refresh(self._h)

    def quench(self):
        self._L.oq_quench(self._h)

    def timeStep(self):
        self._check(self._L.oq_time_step(self._h))

    def timeSteps(self, n):
        self._check(self._L.oq_time_steps(self._h, int(n)))

    def flowSteps(self, n, v_frame):
        self._check(self._L.oq_flow_steps(self._h, int(n), float(v_frame)))

    def timeStepsUntilEvent(self, tol=1e-5, niter_tol=10, max_iter=int(1e9)):
        r = ctypes.c_uint64()
        self._check(self._L.oq_time_steps_until_event(self._h, tol, niter_tol, max_iter, ctypes.byref(r)))
        return r.value

    def minimise(self, tol=1e-5, niter_tol=10, max_iter=int(1e9), time_activity=False, max_iter_is_error=True):
        r = ctypes.c_uint64()
        self._check(self._L.oq_minimise(self._h, tol, niter_tol, int(max_iter), int(time_activity),
                                      int(max_iter_is_error), ctypes.byref(r)))
        return r.value

    @property
    def f_thermal(self):
        out = np.empty(self.size)
        self._check(self._L.oq_get_thermal(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out.reshape(self.shape)

    @f_thermal.setter
    def f_thermal(self, value):
        a = np.ascontiguousarray(np.broadcast_to(value, self.shape), dtype=np.float64).ravel()
        self._check(self._L.oq_thermal_set(self._h, None, a.ctypes.data, None))

    @property
    def thermal_state(self):
        out = ctypes.c_uint64()
        self._check(self._L.oq_thermal_get(self._h, ctypes.addressof(out), None, None))
        return out.value

    @thermal_state.setter
    def thermal_state(self, value):
        st = ctypes.c_uint64(int(value))
        self._check(self._L.oq_thermal_set(self._h, ctypes.addressof(st), None, None))

    @property
    def thermal_next(self):
        out = np.empty(self.size, np.int64)
        self._check(self._L.oq_thermal_get(self._h, None, None, out.ctypes.data))
        return out.reshape(self.shape)

    @thermal_next.setter
    def thermal_next(self, value):
        a = np.ascontiguousarray(np.broadcast_to(value, self.shape), dtype=np.int64).ravel()
        self._check(self._L.oq_thermal_set(self._h, None, None, a.ctypes.data))

    def minimise_nopassing(self, tol=1e-5, niter_tol=10, max_iter=int(1e9), max_iter_is_error=True):
        r = ctypes.c_uint64()
        self._check(self._L.oq_minimise_nopassing(self._h, tol, niter_tol, int(max_iter), int(max_iter_is_error),
                                                ctypes.byref(r)))
        return r.value

    def minimise_truncate(self, i_n, A_truncate=0, S_truncate=0, tol=1e-5, niter_tol=10, max_iter=int(1e9),
                          time_activity=True, max_iter_is_error=True):
        idx = np.ascontiguousarray(i_n, dtype=np.int64).ravel()
        r = ctypes.c_uint64()
        self._check(self._L.oq_minimise_truncate(self._h, _ptr(idx), A_truncate, S_truncate, tol, niter_tol,
                                               int(max_iter), int(time_activity), int(max_iter_is_error),
                                               ctypes.byref(r)))
        return r.value

    def maxUniformDisplacement(self, direction=1):
        r = ctypes.c_double()
        self._check(self._L.oq_max_uniform_displacement(self._h, direction, ctypes.byref(r)))
        return r.value

    def eventDrivenStep(self, eps, kick, direction=1):
        r = ctypes.c_double()
        self._check(self._L.oq_event_driven_step(self._h, eps, int(kick), direction, ctypes.byref(r)))
        return r.value

    def trigger(self, p, eps, direction=1):
        self._check(self._L.oq_trigger(self._h, int(p), eps, direction))

    def advanceToFixedForce(self, f_frame, allow_plastic=False):
        self._check(self._L.oq_advance_to_fixed_force(self._h, f_frame, int(allow_plastic)))

    def yield_sequence(self, p, k0, count):
        out = np.empty(count)
        self._check(self._L.oq_yield_sequence(self._h, p, k0, count, _ptr(out)))
        return out


def line1d(potential="Cuspy", **kw):
    pot = {"Cuspy": CUSPY, "SemiSmooth": SEMISMOOTH, "Smooth": SMOOTH}[potential]
    return System(pot, LAPLACE1D, **kw)


def line1d_nopassing(mu, k_interactions, k_frame, shape, seed, distribution, parameters, offset=-100.0,
                     nchunk=5000, eta=0.0, dt=0.0, **kw):
    """System_Cuspy_Laplace_Nopassing (Line1d.h:173-238): Cuspy + Laplace1d with m = 1; minimise it with
    `minimise_nopassing` (the reference's class has no dynamics)."""
    return System(CUSPY, LAPLACE1D, m=1.0, eta=eta, mu=mu, k_interactions=k_interactions, k_frame=k_frame, dt=dt,
                  shape=shape, seed=seed, distribution=distribution, parameters=parameters, offset=offset,
                  nchunk=nchunk, **kw)


def line1d_quartic(m, eta, mu, a1, a2, k_frame, dt, shape, seed, distribution, parameters, **kw):
    """System_Cuspy_Quartic (Line1d.h:428-481)."""
    return System(CUSPY, QUARTIC1D, shape=shape, m=m, eta=eta, mu=mu, k_interactions=0.0, k_frame=k_frame, dt=dt,
                  seed=seed, distribution=distribution, parameters=parameters, interaction_parameters=(a1, a2), **kw)


def line1d_quartic_gradient(m, eta, mu, k2, k4, k_frame, dt, shape, seed, distribution, parameters, **kw):
    """Line1d System_Cuspy_QuarticGradient (Line1d.h:562-615)."""
    return System(CUSPY, QUARTICGRAD1D, shape=shape, m=m, eta=eta, mu=mu, k_interactions=0.0, k_frame=k_frame,
                  dt=dt, seed=seed, distribution=distribution, parameters=parameters, interaction_parameters=(k2, k4),
                  **kw)


def line2d_quartic_gradient(m, eta, mu, k2, k4, k_frame, dt, shape, seed, distribution, parameters, **kw):
    """Line2d System_Cuspy_QuarticGradient (Line2d.h:122-167)."""
    return System(CUSPY, QUARTICGRAD2D, shape=shape, m=m, eta=eta, mu=mu, k_interactions=0.0, k_frame=k_frame,
                  dt=dt, seed=seed, distribution=distribution, parameters=parameters, interaction_parameters=(k2, k4),
                  **kw)


def line1d_longrange(m, eta, mu, k_interactions, alpha, k_frame, dt, shape, seed, distribution, parameters, **kw):
    """System_Cuspy_LongRange (Line1d.h:617-675, LongRange1d detail.h:812-868)."""
    return System(CUSPY, LONGRANGE1D, shape=shape, m=m, eta=eta, mu=mu, k_interactions=k_interactions,
                  k_frame=k_frame, dt=dt, seed=seed, distribution=distribution, parameters=parameters,
                  interaction_parameters=(alpha, 0.0), **kw)


PCG32_DEFAULT_STREAM = 0xDA3E39CB94B95BDB  # prrng's pcg32(seed) stream (pinned by the RandomForcing golden)
_M64 = (1 << 64) - 1
_PCG_MULT = 0x5851F42D4C957F2D


def pcg32_seed(initstate, initseq=PCG32_DEFAULT_STREAM):
    """(state, inc) of pcg32 seeded with (initstate, initseq) (the PCG seeding procedure)."""
    inc = ((initseq << 1) | 1) & _M64
    state = inc  # 0 * mult + inc
    state = (state + initstate) & _M64
    state = (state * _PCG_MULT + inc) & _M64
    return state, inc


def pcg32_randint(seed, n, high, initseq=PCG32_DEFAULT_STREAM):
    """n draws in [0, high) as prrng.pcg32(seed).randint([n], high): the PCG bounded draw (reject
    u32 below (2^32 - high) % high, then u32 % high).  Pinned with pcg32_seed's default stream by the
    reference's RandomForcing golden trajectory."""
    state, inc = pcg32_seed(seed, initseq)
    thr = ((1 << 32) - high) % high
    out = np.empty(n, dtype=np.int64)
    i = 0
    while i < n:
        old = state
        state = (old * _PCG_MULT + inc) & _M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        r = ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF
        if r >= thr:
            out[i] = r % high
            i += 1
    return out


def attach_random_forcing(s, mean, stddev, seed_forcing, dinc_init, dinc):
    """RandomNormalForcing (detail.h:881-1000) on an oracle system, drawn at its current inc as the
    RandomForcing constructors' refresh does."""
    n = s.size
    s._th_next = np.ascontiguousarray(np.broadcast_to(dinc_init, (n,)), dtype=np.int64)
    s._th_dinc = np.ascontiguousarray(np.broadcast_to(dinc, (n,)), dtype=np.int64)
    state, inc = pcg32_seed(int(seed_forcing))
    s._check(s._L.oq_set_thermal(s._h, float(mean), float(stddev), state, inc, s._th_next.ctypes.data,
                                  s._th_dinc.ctypes.data, 0))
    return s


def line1d_random_forcing(m, eta, mu, k_interactions, k_frame, dt, mean, stddev, seed_forcing, dinc_init, dinc,
                          shape, seed, distribution, parameters, offset=-100.0, nchunk=5000, **kw):
    """System_Cuspy_Laplace_RandomForcing (Line1d.h:264-330, RandomNormalForcing detail.h:881-1000):
    every `dinc` increments (first at `dinc_init`) a particle's thermal force is redrawn from one pcg32
    stream (seed_forcing, prrng's default stream), in particle order, as mean + stddev sqrt(2)
    erfinv(2 r - 1), r = u32 2^-32."""
    s = System(CUSPY, LAPLACE1D, shape=shape, m=m, eta=eta, mu=mu, k_interactions=k_interactions, k_frame=k_frame,
               dt=dt, seed=seed, distribution=distribution, parameters=parameters, offset=offset, nchunk=nchunk,
               **kw)
    return attach_random_forcing(s, mean, stddev, seed_forcing, dinc_init, dinc)


def line2d(**kw):
    return System(CUSPY, LAPLACE2D, **kw)


def particles(potential="Cuspy", **kw):
    pot = {"Cuspy": CUSPY, "SemiSmooth": SEMISMOOTH, "Smooth": SMOOTH}[potential]
    kw.setdefault("k_interactions", 0.0)
    return System(pot, NONE, **kw)
