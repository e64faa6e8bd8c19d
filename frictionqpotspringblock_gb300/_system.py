"""Python classes of the drop-in API, over the C ABI (include/fqsb.h).

Names, argument names and defaults follow the reference's pybind11 module
(python/main.cpp:46-226 in the reference project):

* mySystemNd          main.cpp:46-156   properties and state setters
* mySystemNdAthermal  main.cpp:158-202  minimise, minimise_truncate, eventDrivenStep
* mySystemNdDynamics  main.cpp:210-226  timeStep, timeSteps, timeStepsUntilEvent, flowSteps

One documented divergence: getters return numpy snapshots (copies from the
device), not live views of the state; `system.u += du` still works because
Python calls the setter with the updated array.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _capi as C


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


class Chunk:
    """Proxy of the prrng chunk (`system.chunk`) with the member names the reference's tests use."""

    def __init__(self, system: "System"):
        self._s = system

    def _index(self, which: int):
        s = self._s
        n = s.size
        out = np.empty(n, np.int64) if which < 2 else np.empty(n, np.float64)
        args = [None, None, None, None]
        args[which] = _ptr(out, ctypes.c_int64 if which < 2 else ctypes.c_double)
        C.check(s._h, C.lib().fqsb_get_index(s._h, *args))
        return out.reshape(s.shape)

    @property
    def index_at_align(self) -> np.ndarray:
        """Global index i of the current well: y[i] <= u < y[i + 1]."""
        return self._index(0)

    @property
    def chunk_index_at_align(self) -> np.ndarray:
        return self._index(1)

    @property
    def left_of_align(self) -> np.ndarray:
        return self._index(2)

    @property
    def right_of_align(self) -> np.ndarray:
        return self._index(3)

    @property
    def chunk_size(self) -> int:
        return self._s.nchunk

    @property
    def data(self) -> np.ndarray:
        s = self._s
        out = np.empty(s.size * s.nchunk)
        C.check(s._h, C.lib().fqsb_chunk_data(s._h, _ptr(out, ctypes.c_double), None))
        return out.reshape(tuple(s.shape) + (s.nchunk,))

    @property
    def start(self) -> np.ndarray:
        s = self._s
        out = np.empty(s.size, np.int64)
        C.check(s._h, C.lib().fqsb_chunk_data(s._h, None, _ptr(out, ctypes.c_int64)))
        return out.reshape(s.shape)

    def state_at(self, index) -> np.ndarray:
        s = self._s
        idx = np.ascontiguousarray(np.broadcast_to(index, s.shape), dtype=np.int64).ravel()
        out = np.empty(s.size, np.uint64)
        C.check(s._h, C.lib().fqsb_chunk_state_at(s._h, _ptr(idx, ctypes.c_int64), _ptr(out, ctypes.c_uint64)))
        return out.reshape(s.shape)

    def restore(self, state, value, index):
        s = self._s
        st = np.ascontiguousarray(np.broadcast_to(state, s.shape), dtype=np.uint64).ravel()
        val = np.ascontiguousarray(np.broadcast_to(value, s.shape), dtype=np.float64).ravel()
        idx = np.ascontiguousarray(np.broadcast_to(index, s.shape), dtype=np.int64).ravel()
        C.check(s._h, C.lib().fqsb_chunk_restore(s._h, _ptr(st, ctypes.c_uint64), _ptr(val, ctypes.c_double),
                                                 _ptr(idx, ctypes.c_int64)))


class RandomNormalForcing:
    """Proxy of `system.external` of the RandomForcing systems (detail.RandomNormalForcing_1,
    main.cpp:251-275, detail.h:881-1000): the pcg32 state of the draws, the current thermal forces and
    the increment of each particle's next draw.  Getters return copies; setters write through."""

    def __init__(self, system: "System"):
        self._s = system

    def __repr__(self):
        return "<FrictionQPotSpringBlock.detail.RandomNormalForcing_1>"

    @property
    def state(self) -> int:
        """State of RNG"""
        s = self._s
        out = ctypes.c_uint64()
        C.check(s._h, C.lib().fqsb_random_forcing_get(s._h, ctypes.byref(out), None, None))
        return out.value

    @state.setter
    def state(self, value):
        s = self._s
        st = ctypes.c_uint64(int(value))
        C.check(s._h, C.lib().fqsb_random_forcing_set(s._h, ctypes.byref(st), None, None))

    @property
    def f_thermal(self) -> np.ndarray:
        """Random force"""
        s = self._s
        out = np.empty(s.size)
        C.check(s._h, C.lib().fqsb_random_forcing_get(s._h, None, _ptr(out, ctypes.c_double), None))
        return out.reshape(s.shape)

    @f_thermal.setter
    def f_thermal(self, value):
        s = self._s
        arr = np.ascontiguousarray(value, dtype=np.float64)
        if list(arr.shape) != s.shape:
            raise RuntimeError("assertion failed (xt::has_shape(f_thermal, m_f_thermal.shape()))")
        arr = arr.ravel()
        C.check(s._h, C.lib().fqsb_random_forcing_set(s._h, None, _ptr(arr, ctypes.c_double), None))

    @property
    def next(self) -> np.ndarray:
        """Next draw increment"""
        s = self._s
        out = np.empty(s.size, np.int64)
        C.check(s._h, C.lib().fqsb_random_forcing_get(s._h, None, None, _ptr(out, ctypes.c_int64)))
        return out.reshape(s.shape)

    @next.setter
    def next(self, value):
        s = self._s
        arr = np.ascontiguousarray(value, dtype=np.int64)
        if list(arr.shape) != s.shape:
            raise RuntimeError("assertion failed (xt::has_shape(next, m_next.shape()))")
        arr = arr.ravel()
        C.check(s._h, C.lib().fqsb_random_forcing_set(s._h, None, None, _ptr(arr, ctypes.c_int64)))


class _Hidden:
    """A member of the base class that this class does not have (raises AttributeError, hasattr is False)."""

    def __set_name__(self, owner, name):
        self._name = name

    def __get__(self, obj, objtype=None):
        raise AttributeError(f"'{objtype.__name__}' object has no attribute '{self._name}'")


class System:
    """A system resident on the GPU.  Concrete classes fix the potential and the interactions."""

    _potential = C.CUSPY
    _interactions = C.LAPLACE1D
    _rank = 1
    _name = "System"

    def __init__(self, m, eta, mu, k_interactions, k_frame, dt, shape, seed, distribution, parameters,
                 offset=-100.0, nchunk=5000, kappa=0.0, offset_per_particle=None, stream=None, device=0,
                 interaction_parameters=(0.0, 0.0)):
        shape = [int(i) for i in np.atleast_1d(shape)]
        if len(shape) != self._rank:
            raise ValueError(f"shape must have {self._rank} entries")
        rows, cols = (1, shape[0]) if self._rank == 1 else (shape[0], shape[1])
        if distribution not in C.DISTRIBUTIONS:
            raise RuntimeError("Unknown distribution: " + str(distribution))
        parameters = [float(p) for p in parameters]
        if len(parameters) > 4:
            raise ValueError("at most 4 distribution parameters")
        cfg = C.Config()
        cfg.potential = self._potential
        cfg.interactions = self._interactions
        cfg.rows, cfg.cols = rows, cols
        cfg.m, cfg.eta, cfg.mu, cfg.kappa = float(m), float(eta), float(mu), float(kappa)
        cfg.k_interactions, cfg.k_frame, cfg.dt = float(k_interactions), float(k_frame), float(dt)
        cfg.interaction_parameters[0] = float(interaction_parameters[0])
        cfg.interaction_parameters[1] = float(interaction_parameters[1])
        cfg.seed = int(seed)
        cfg.distribution = C.DISTRIBUTIONS[distribution]
        cfg.n_parameters = len(parameters)
        for i, p in enumerate(parameters):
            cfg.parameters[i] = p
        cfg.offset = float(offset)
        self._offp = None
        if offset_per_particle is not None:
            self._offp = np.ascontiguousarray(np.broadcast_to(offset_per_particle, shape), dtype=np.float64).ravel()
            cfg.offset_per_particle = _ptr(self._offp, ctypes.c_double)
        cfg.nchunk = int(nchunk)
        cfg.stream = stream
        cfg.device = int(device)
        h = ctypes.c_void_p()
        status = C.lib().fqsb_create(ctypes.byref(cfg), ctypes.byref(h))
        if status != C.OK:
            raise C.FrictionError(status, C.lib().fqsb_last_error(None).decode())
        self._h = h
        self._device = int(device)
        self._shape = shape
        self._size = rows * cols
        self._nchunk = int(nchunk)
        self._dt, self._mu, self._eta, self._m, self._k_frame = float(dt), float(mu), float(eta), float(m), float(k_frame)
        self._chunk = Chunk(self)

    def _attach_random_forcing(self, mean, stddev, seed_forcing, dinc_init, dinc):
        """RandomNormalForcing of the RandomForcing systems (detail.h:903-919), attached at construction."""
        self._th_next0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dinc_init), self._shape), dtype=np.int64)
        self._th_dinc = np.ascontiguousarray(np.broadcast_to(np.asarray(dinc), self._shape), dtype=np.int64)
        C.check(self._h, C.lib().fqsb_set_random_forcing(self._h, float(mean), float(stddev), int(seed_forcing),
                                                          _ptr(self._th_next0.ravel(), ctypes.c_int64),
                                                          _ptr(self._th_dinc.ravel(), ctypes.c_int64)))
        self._external = RandomNormalForcing(self)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            C.lib().fqsb_destroy(h)
            self._h = None

    def __repr__(self):
        return f"<FrictionQPotSpringBlock.{self._name}>"

    # ---------------------------------------------------------------- parameters
    chunk = property(lambda s: s._chunk, doc="Chunk of random numbers")
    size = property(lambda s: s._size, doc="Number of particles")
    shape = property(lambda s: list(s._shape), doc="Shape of the system")
    dt = property(lambda s: s._dt, doc="Time step (parameter)")
    mu = property(lambda s: s._mu, doc="Curvature of each well (parameter)")
    eta = property(lambda s: s._eta, doc="Damping coefficient (parameter)")
    m = property(lambda s: s._m, doc="Mass of each particle (parameter)")
    k_frame = property(lambda s: s._k_frame, doc="Loading frame stiffness (parameter)")
    nchunk = property(lambda s: s._nchunk)

    # deprecated names (main.cpp:49-63)
    @property
    def x(self):
        raise RuntimeError("Deprecated, use 'u'")

    @x.setter
    def x(self, value):
        raise RuntimeError("Deprecated, use 'u'")

    @property
    def x_frame(self):
        raise RuntimeError("Deprecated, use 'u_frame'")

    @x_frame.setter
    def x_frame(self, value):
        raise RuntimeError("Deprecated, use 'u_frame'")

    @property
    def f_neighbours(self):
        raise RuntimeError("Deprecated, use 'f_interactions'")

    # ---------------------------------------------------------------- fields
    def _get(self, field: int) -> np.ndarray:
        out = np.empty(self._size)
        C.check(self._h, C.lib().fqsb_get_field(self._h, field, _ptr(out, ctypes.c_double)))
        return out.reshape(self._shape)

    def _set(self, field: int, value):
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(value, dtype=np.float64), self._shape)).ravel()
        C.check(self._h, C.lib().fqsb_set_field(self._h, field, _ptr(arr, ctypes.c_double)))

    u = property(lambda s: s._get(C.FIELD_U), lambda s, x: s._set(C.FIELD_U, x), doc="Particle slip ('positions').")
    v = property(lambda s: s._get(C.FIELD_V), lambda s, x: s._set(C.FIELD_V, x), doc="Particle velocities.")
    a = property(lambda s: s._get(C.FIELD_A), lambda s, x: s._set(C.FIELD_A, x), doc="Particle accelerations.")
    f = property(lambda s: s._get(C.FIELD_F), doc="Residual forces")
    f_potential = property(lambda s: s._get(C.FIELD_F_POTENTIAL), doc="Elastic forces")
    f_frame = property(lambda s: s._get(C.FIELD_F_FRAME), doc="Frame forces")
    f_interactions = property(lambda s: s._get(C.FIELD_F_INTERACTIONS), doc="Interaction forces")
    f_damping = property(lambda s: s._get(C.FIELD_F_DAMPING), doc="Particle damping forces")

    def _scalar(self, which: int) -> float:
        out = ctypes.c_double()
        C.check(self._h, C.lib().fqsb_get_scalar(self._h, which, ctypes.byref(out)))
        return out.value

    temperature = property(lambda s: s._scalar(C.SCALAR_TEMPERATURE), doc="Temperature")
    residual = property(lambda s: s._scalar(C.SCALAR_RESIDUAL), doc="Residual")

    @property
    def u_frame(self) -> float:
        return self._scalar(C.SCALAR_U_FRAME)

    @u_frame.setter
    def u_frame(self, value):
        C.check(self._h, C.lib().fqsb_set_u_frame(self._h, float(value)))

    @property
    def inc(self) -> int:
        out = ctypes.c_int64()
        C.check(self._h, C.lib().fqsb_get_inc(self._h, ctypes.byref(out)))
        return out.value

    @inc.setter
    def inc(self, value):
        C.check(self._h, C.lib().fqsb_set_inc(self._h, int(value)))

    @property
    def t(self) -> float:
        return self._scalar(C.SCALAR_T)

    @t.setter
    def t(self, value):
        C.check(self._h, C.lib().fqsb_set_t(self._h, float(value)))

    # convenience names of the current well (the changelog's i / y_left / y_right)
    i = property(lambda s: s._chunk.index_at_align)
    y_left = property(lambda s: s._chunk.left_of_align)
    y_right = property(lambda s: s._chunk.right_of_align)

    @property
    def quasistaticActivityFirst(self) -> int:
        a, b = ctypes.c_int64(), ctypes.c_int64()
        C.check(self._h, C.lib().fqsb_quasistatic_activity(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value

    @property
    def quasistaticActivityLast(self) -> int:
        a, b = ctypes.c_int64(), ctypes.c_int64()
        C.check(self._h, C.lib().fqsb_quasistatic_activity(self._h, ctypes.byref(a), ctypes.byref(b)))
        return b.value

    # ---------------------------------------------------------------- methods
    def refresh(self):
        C.check(self._h, C.lib().fqsb_refresh(self._h))

    def quench(self):
        C.check(self._h, C.lib().fqsb_quench(self._h))

    def maxUniformDisplacement(self, direction=1) -> float:
        out = ctypes.c_double()
        C.check(self._h, C.lib().fqsb_max_uniform_displacement(self._h, int(direction), ctypes.byref(out)))
        return out.value

    def trigger(self, p, eps, direction=1):
        C.check(self._h, C.lib().fqsb_trigger(self._h, int(p), float(eps), int(direction)))

    def advanceToFixedForce(self, f_frame, allow_plastic=False):
        C.check(self._h, C.lib().fqsb_advance_to_fixed_force(self._h, float(f_frame), int(bool(allow_plastic))))

    def minimise(self, tol=1e-5, niter_tol=10, max_iter=int(1e9), time_activity=False, max_iter_is_error=True) -> int:
        out = ctypes.c_uint64()
        C.check(self._h, C.lib().fqsb_minimise(self._h, float(tol), int(niter_tol), int(max_iter), int(bool(time_activity)),
                                               int(bool(max_iter_is_error)), ctypes.byref(out)))
        return out.value

    def minimise_truncate(self, i_n, A_truncate=0, S_truncate=0, tol=1e-5, niter_tol=10, max_iter=int(1e9),
                          time_activity=True, max_iter_is_error=True) -> int:
        idx = np.ascontiguousarray(np.broadcast_to(i_n, self._shape), dtype=np.int64).ravel()
        out = ctypes.c_uint64()
        C.check(self._h, C.lib().fqsb_minimise_truncate(self._h, _ptr(idx, ctypes.c_int64), int(A_truncate),
                                                        int(S_truncate), float(tol), int(niter_tol), int(max_iter),
                                                        int(bool(time_activity)), int(bool(max_iter_is_error)),
                                                        ctypes.byref(out)))
        return out.value

    def eventDrivenStep(self, eps, kick, direction=1) -> float:
        out = ctypes.c_double()
        C.check(self._h, C.lib().fqsb_event_driven_step(self._h, float(eps), int(bool(kick)), int(direction),
                                                        ctypes.byref(out)))
        return out.value

    def timeStep(self):
        C.check(self._h, C.lib().fqsb_time_step(self._h))

    def timeSteps(self, n):
        C.check(self._h, C.lib().fqsb_time_steps(self._h, int(n)))

    def timeStepsUntilEvent(self, tol=1e-5, niter_tol=10, max_iter=int(1e9)) -> int:
        out = ctypes.c_uint64()
        C.check(self._h, C.lib().fqsb_time_steps_until_event(self._h, float(tol), int(niter_tol), int(max_iter),
                                                             ctypes.byref(out)))
        return out.value

    def flowSteps(self, n, v_frame):
        C.check(self._h, C.lib().fqsb_flow_steps(self._h, int(n), float(v_frame)))

    # ---------------------------------------------------------------- differentiation support
    def set_parameters(self, mu, k_interactions, eta):
        """Change mu, k_interactions and eta of the existing system (an extension; the reference fixes
        them at construction)."""
        C.check(self._h, C.lib().fqsb_set_parameters(self._h, float(mu), float(k_interactions), float(eta)))
        self._mu, self._eta = float(mu), float(eta)

    def adjoint_forward(self, schedule, K=100, last=500) -> float:
        """From the current state run len(schedule) steps with u_frame = schedule[t] set before step t,
        keeping checkpoints every K steps; returns
        L = mean over the last `last` steps of mean(f_frame) + 0.5 * mean(u_T**2)."""
        sched = np.ascontiguousarray(schedule, dtype=np.float64)
        loss = ctypes.c_double()
        C.check(self._h, C.lib().fqsb_adjoint_forward(self._h, _ptr(sched, ctypes.c_double), len(sched), int(K),
                                                      int(last), ctypes.byref(loss)))
        self._adj_T = len(sched)
        return loss.value

    def adjoint_backward(self):
        """Gradients of the last adjoint_forward's loss: (dL/du0, dL/dv0, dL/dschedule,
        [dL/dmu, dL/dk_interactions, dL/deta])."""
        gu = np.empty(self._size)
        gv = np.empty(self._size)
        gs = np.empty(self._adj_T)
        gp = np.empty(3)
        C.check(self._h, C.lib().fqsb_adjoint_backward(self._h, _ptr(gu, ctypes.c_double), _ptr(gv, ctypes.c_double),
                                                       _ptr(gs, ctypes.c_double), _ptr(gp, ctypes.c_double)))
        return gu.reshape(self._shape), gv.reshape(self._shape), gs, gp

    def adjoint_backward_device(self, grad_u0_ptr: int, grad_v0_ptr: int):
        """As adjoint_backward, with dL/du0 and dL/dv0 written to device arrays of N doubles on the system's
        device (pointers as integers); returns (dL/dschedule, [dL/dmu, dL/dk_interactions, dL/deta])."""
        gs = np.empty(self._adj_T)
        gp = np.empty(3)
        C.check(self._h, C.lib().fqsb_adjoint_backward_device(self._h, ctypes.c_void_p(grad_u0_ptr),
                                                              ctypes.c_void_p(grad_v0_ptr),
                                                              _ptr(gs, ctypes.c_double), _ptr(gp, ctypes.c_double)))
        return gs, gp

    # ---------------------------------------------------------------- device access
    @property
    def device(self) -> int:
        """The CUDA device ordinal the system lives on."""
        return self._device

    @property
    def stream(self) -> int:
        """The cudaStream_t (as an integer) the system launches its kernels on."""
        out = ctypes.c_void_p()
        C.check(self._h, C.lib().fqsb_get_stream(self._h, ctypes.byref(out)))
        return out.value or 0

    def get_field_device(self, field: int, device_ptr: int):
        C.check(self._h, C.lib().fqsb_get_field_device(self._h, field, ctypes.c_void_p(device_ptr)))

    def set_field_device(self, field: int, device_ptr: int):
        C.check(self._h, C.lib().fqsb_set_field_device(self._h, field, ctypes.c_void_p(device_ptr)))
