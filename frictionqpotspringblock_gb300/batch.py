"""Batched form: many independent Line1d System_Cuspy_Laplace realisations on one GPU.

The reference runs one System at a time; this form runs thousands of disorder realisations of uneven
size together -- one graph launch for a whole quasistatic protocol, each realisation converging on its
own (include/fqsb.h, fqsb_batch_*).  Every realisation follows exactly the arithmetic of the plain
path, so its trajectory and well indices are those of
`Line1d.System_Cuspy_Laplace(...)` driven by `eventDrivenStep(eps, False)`,
`eventDrivenStep(eps, True)`, `minimise(tol)` in a loop.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _capi as C


def pcg32_uniform(seed: int, n: int, initseq: int = 0) -> np.ndarray:
    """n uniform draws u32 * 2^-32 of pcg32(initstate=seed, initseq) -- the realisation-size stream."""
    mask = (1 << 64) - 1
    mult = 0x5851F42D4C957F2D
    inc = ((initseq << 1) | 1) & mask
    state = (inc) & mask  # state = 0 * mult + inc
    state = (state + seed) & mask
    state = (state * mult + inc) & mask
    out = np.empty(n)
    for i in range(n):
        old = state
        state = (old * mult + inc) & mask
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        r = ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF
        out[i] = r * 2.0 ** -32
    return out


def log_uniform_sizes(n_instances: int = 4096, lo: int = 256, hi: int = 65536, seed: int = 3) -> np.ndarray:
    """Realisation sizes N_j = round(exp(U(ln lo, ln hi))) with U from pcg32(seed)."""
    u = pcg32_uniform(seed, n_instances)
    a, b = math.log(lo), math.log(hi)
    return np.rint(np.exp(a + u * (b - a))).astype(np.int64)


def partition(sizes, world: int):
    """Split realisations over `world` ranks with no exchange between them: longest-processing-time
    greedy on the sizes (largest first, each to the rank with the least total so far; ties to the
    lowest rank).  Returns one sorted index array per rank; every realisation appears exactly once.
    A rank builds its batch from sizes[idx], seeds[idx] and runs independently; results are placed
    back by idx (weak scaling: no collective on the data path)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(len(sizes), dtype=np.int64)
    for j in order:
        r = int(np.argmin(load))
        owner[j] = r
        load[r] += sizes[j]
    return [np.flatnonzero(owner == r) for r in range(world)]


class Line1d_System_Cuspy_Laplace:
    """A batch of independent Line1d System_Cuspy_Laplace realisations.

    sizes[j], seeds[j], k_frame[j] per realisation (k_frame may be a scalar); the other parameters
    are shared and have the reference constructor's meaning (main.cpp:493-520).  `window` yield
    positions are kept per particle (34 <= window <= nchunk); `threads` x `ppt` is the CTA tile
    (0: default, see autotune.choose_tile)."""

    def __init__(self, sizes, seeds, k_frame, m, eta, mu, k_interactions, dt, distribution, parameters,
                 offset=-100.0, nchunk=5000, window=64, threads=0, ppt=0, device=0):
        self._sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        n = len(self._sizes)
        self._seeds = np.ascontiguousarray(np.broadcast_to(seeds, (n,)), dtype=np.uint64)
        self._kf = np.ascontiguousarray(np.broadcast_to(k_frame, (n,)), dtype=np.float64)
        parameters = [float(p) for p in parameters]
        cfg = C.BatchConfig()
        cfg.n_instances = n
        cfg.sizes = self._sizes.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        cfg.seeds = self._seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        cfg.k_frame = self._kf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        cfg.m, cfg.eta, cfg.mu, cfg.k_interactions, cfg.dt = float(m), float(eta), float(mu), float(k_interactions), float(dt)
        cfg.distribution = C.DISTRIBUTIONS[distribution]
        cfg.n_parameters = len(parameters)
        for i, p in enumerate(parameters):
            cfg.parameters[i] = p
        cfg.offset = float(offset)
        cfg.nchunk = int(nchunk)
        cfg.window = int(min(window, nchunk))
        cfg.threads = int(threads)
        cfg.ppt = int(ppt)
        cfg.stream = None
        cfg.device = int(device)
        h = ctypes.c_void_p()
        st = C.lib().fqsb_batch_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != C.OK:
            raise C.FrictionError(st, C.lib().fqsb_batch_last_error(None).decode())
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            C.lib().fqsb_batch_destroy(h)
            self._h = None

    def _check(self, st):
        if st != C.OK:
            raise C.FrictionError(st, C.lib().fqsb_batch_last_error(self._h).decode())

    @property
    def sizes(self) -> np.ndarray:
        return self._sizes.copy()

    def quasistatic(self, ncycles, eps, tol=1e-5, niter_tol=10, max_iter=int(1e9)):
        """Run ncycles cycles of eventDrivenStep(eps, False), eventDrivenStep(eps, True), minimise(tol)
        on every realisation.  Returns per-cycle arrays [n_instances, ncycles]: u_frame, f_frame (mean),
        S (sum of well-index changes), inc, and the per-realisation status (0 = converged every cycle)."""
        n = len(self._sizes)
        uf = np.empty((n, ncycles))
        ff = np.empty((n, ncycles))
        S = np.empty((n, ncycles), np.int64)
        inc = np.empty((n, ncycles), np.int64)
        status = np.empty(n, np.int32)
        P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
        self._check(C.lib().fqsb_batch_quasistatic(self._h, int(ncycles), float(eps), float(tol), int(niter_tol),
                                                   int(max_iter), P(uf, ctypes.c_double), P(ff, ctypes.c_double),
                                                   P(S, ctypes.c_int64), P(inc, ctypes.c_int64),
                                                   P(status, ctypes.c_int32)))
        return {"u_frame": uf, "f_frame": ff, "S": S, "inc": inc, "status": status}

    def field(self, j: int, name: str = "u") -> np.ndarray:
        fid = {"u": C.FIELD_U, "v": C.FIELD_V, "a": C.FIELD_A}[name]
        out = np.empty(int(self._sizes[j]))
        self._check(C.lib().fqsb_batch_get(self._h, int(j), fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def index_at_align(self, j: int) -> np.ndarray:
        out = np.empty(int(self._sizes[j]), np.int64)
        self._check(C.lib().fqsb_batch_get_index(self._h, int(j), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    @property
    def u_frame(self) -> np.ndarray:
        out = np.empty(len(self._sizes))
        self._check(C.lib().fqsb_batch_frame(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out


def quasistatic_shard(sizes, seeds, k_frame, rank: int, world: int, ncycles: int, eps: float, tol: float = 1e-5,
                      niter_tol: int = 10, max_iter: int = int(1e9), device: int = 0, **kwargs):
    """One rank's part of a sharded batch: the realisations partition(sizes, world)[rank] as one batch on
    `device`, run through `ncycles` quasistatic cycles.  Returns (idx, result) with result as
    Line1d_System_Cuspy_Laplace.quasistatic gives it for those realisations (rows in idx order).  The
    ranks exchange nothing while they run: gathering the per-realisation results (by idx) is the
    caller's, e.g. with torch.distributed.all_gather_object.  kwargs: the shared constructor
    parameters of Line1d_System_Cuspy_Laplace."""
    sizes = np.asarray(sizes, dtype=np.int64)
    seeds = np.asarray(np.broadcast_to(seeds, sizes.shape), dtype=np.uint64)
    k_frame = np.asarray(np.broadcast_to(k_frame, sizes.shape), dtype=np.float64)
    idx = partition(sizes, world)[rank]
    if len(idx) == 0:
        empty = np.empty((0, ncycles))
        return idx, {"u_frame": empty, "f_frame": empty, "S": empty.astype(np.int64), "inc": empty.astype(np.int64),
                     "status": np.empty(0, np.int32)}
    b = Line1d_System_Cuspy_Laplace(sizes[idx], seeds[idx], k_frame[idx], device=device, **kwargs)
    out = b.quasistatic(ncycles, eps, tol=tol, niter_tol=niter_tol, max_iter=max_iter)
    del b
    return idx, out
