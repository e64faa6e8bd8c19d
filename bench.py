"""Benchmark of the GB300 time-integration path (and of the CPU reference arm).

Workload (the large-N throughput configuration): Line1d System_Cuspy_Laplace,
N = 2^22 particles on a periodic ring, m = 1, eta = 0.1, mu = 1,
k_interactions = 1, k_frame = 1/N, dt = 0.1; yield distances Weibull(k=2,
scale=1) + 1e-5 from pcg32 (seed 1, particle p on stream initstate = 1 + p),
2000 yield positions per particle; initial u ~ N(0, 0.1^2) (numpy PCG64,
seed 1), v = 0.  The frame is ramped by 1e-4 per time step
(flowSteps with v_frame = 1e-3), then jumps by +0.5, then minimise(tol=1e-5).

One bench step = flowSteps(1000): 1000 fused time steps over all particles,
so --steps 10 covers the configuration's 10^4 steps.  The metric is
particle-steps/s (FP64).  After the timed steps the +0.5 jump and minimise are
run once and their wall time is reported (minimise).

`value` times the device-resident steps (state already in HBM); `e2e` times
the same steps through the public API with host buffers: each step copies u
and v from pinned host memory into the system, runs flowSteps(1000) and reads
u back.  `--impl reference` times the CPU reference path instead: the oracle
(the reference's loop-per-statement integrator restated in C, libm, built with
OpenMP so its per-particle loops run over all host cores with bit-identical
results) on the same N = 2^22 ring, seeds and initial state, each bench step a
bounded number of flowSteps time steps.

`forms` times the other configurations (each records an error instead of
raising): small_system (N = 1024 quasistatic protocol), line2d (2048 x 2048
grid), batched (4096 uneven realisations), adjoint (N = 65536, T = 5000
differentiation with finite-difference checks) and next_rows (the further
interactions, the no-passing minimiser, the thermal forcing).  By default the
long protocols run shortened (stated in each entry); --full runs them at their
configured sizes; --forms selects a subset.

Multi-GPU (torchrun): the plain path does not shard (one system fits one GPU),
so every rank runs an independent replica (weak scaling); value = sum of the
ranks' particle-steps / max rank time.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_DEFAULT = 2 ** 22
INNER = 1000
METRIC = "particle-steps/s (FP64)"
PAR = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, seed=1, distribution="weibull",
           parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=2000)
V_FRAME = 1e-3  # u_frame += v_frame * dt = 1e-4 per step
BYTES_PER_PARTICLE_STEP = 64  # read+write u, v, a (48 B) + read the current well {y_left, y_right} (16 B)
FP64_OPS_PER_PARTICLE_STEP = 24  # binary64 add/mul of the exact-order step; compares and 2^k scalings are integer work
# of those, the step kernel issues these on the fp64 pipe; the rest (the 8 multiplications and the 2 additions of
# the position update) run bit-identically on the integer pipes (csrc/fq_soft64.h)
FP64_PIPE_OPS_PER_PARTICLE_STEP = 14
STEP_PROFILE = ROOT / "profiles" / "k_step_line_cuspy_laplace1d_N4M.md"
FORMS = ("small_system", "line2d", "batched", "adjoint", "next_rows")


def workload(n, inner=INNER):
    return (f"Line1d System_Cuspy_Laplace N={n} ring, m=1 eta=0.1 mu=1 k=1 k_frame=1/N dt=0.1, "
            f"weibull(2,1)+1e-5 nchunk=2000 seed=1, u0~N(0,0.1^2); step = flowSteps({inner}, v_frame=1e-3) "
            f"(u_frame +1e-4 per time step); then u_frame += 0.5 and minimise(tol=1e-5)")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_figures(path=STEP_PROFILE):
    """`name = number` lines of a committed profile summary (the ncu figures the roofline uses)."""
    out = {}
    for line in path.read_text().splitlines():
        m = re.fullmatch(r"\s+([a-z_]+) = ([0-9.eE+-]+)", line)
        if m:
            out[m.group(1)] = float(m.group(2))
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in pathlib.Path(self.path).read_text().splitlines():
            cols = [c.strip() for c in line.split(",")]
            if len(cols) < 9:
                continue
            try:
                sm.append(float(cols[1]))
                smax.append(float(cols[2]))
            except ValueError:
                continue
            for name, val in zip(names, cols[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _guard(fn, *a, **kw):
    """A form's failure is recorded in its entry, not raised: the bench line must still be printed."""
    try:
        return fn(*a, **kw)
    except Exception as e:  # noqa: BLE001
        return {"error": f"{type(e).__name__}: {e}"}


def _sync_seconds(t0):
    import torch

    torch.cuda.synchronize()
    return time.perf_counter() - t0


# ------------------------------------------------------------------------------------------ forms

def bench_small(fqsb, full=False, cycles=100, cpu_cycles=100):
    """Small system: Line1d System_Cuspy_Laplace N = 1024, m = 1, eta = 0.1, mu = 1, k = 1,
    k_frame = 1/1024, dt = 0.1, Weibull(2,1)+1e-5 seed 0, 1000-position chunk shifted per particle so
    that u = 0 is the centre of well 500; from u = v = 0, 100 cycles of eventDrivenStep(1e-5,
    kick=False), eventDrivenStep(1e-5, kick=True), minimise(tol=1e-5, max_iter=1e6).  The CPU oracle
    (the reference restated: libm, sequential sums, one core) runs the same protocol.  `sizes`: time
    per time step of timeSteps(20000) and of a minimise after a +0.5 frame jump for N = 64 ... 16384
    (offset -500, nchunk 1000, seed 0), on the one-cluster path and on the CUDA-graph path
    (FQSB_NO_SMALL=1 at construction)."""
    N = 1024
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1, shape=[N], seed=0,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], nchunk=1000)
    plain = fqsb.Line1d.System_Cuspy_Laplace(offset=0.0, **par)
    raw, start = plain.chunk.data, plain.chunk.start  # the window moved so that u = 0 lies inside it
    rows = np.arange(N)
    offp = -0.5 * (raw[rows, 500 - start] + raw[rows, 501 - start])
    del plain

    def run(s, n):
        inc0 = s.inc
        t0 = time.perf_counter()
        for _ in range(n):
            s.eventDrivenStep(1e-5, False)
            s.eventDrivenStep(1e-5, True)
            s.minimise(max_iter=1000000)
        return time.perf_counter() - t0, s.inc - inc0

    s = fqsb.Line1d.System_Cuspy_Laplace(offset=0.0, offset_per_particle=offp, **par)
    assert np.all(s.chunk.index_at_align == 500)
    t_first, steps_first = run(s, 10)
    t_rest, steps_rest = run(s, cycles - 10)
    t, steps = t_first + t_rest, steps_first + steps_rest
    out = {"particles": N, "cycles": cycles, "seconds": t, "seconds_per_cycle": t / cycles, "time_steps": steps,
           "us_per_step": 1e6 * t / steps, "first_10_cycles": {"seconds": t_first, "time_steps": steps_first,
                                                                "us_per_step": 1e6 * t_first / steps_first}}
    if cpu_cycles > 0:
        from oracle import oracle as O  # the CPU baseline: the reference restated, one core

        r = O.line1d("Cuspy", offset=0.0, offset_per_particle=offp, sum_mode=O.SUM_SEQUENTIAL, math_mode=O.MATH_LIBM,
                     **par)
        tc, sc = run(r, cpu_cycles)
        out["cpu_oracle"] = {"cycles": cpu_cycles, "cores": 1, "seconds": tc, "time_steps": sc,
                             "us_per_step": 1e6 * tc / sc}
        if cpu_cycles == cycles:
            out["speedup_vs_cpu_oracle"] = tc / t
    sizes = {}
    for path in ("cluster", "graph"):
        for n in (64, 1024, 4096, 16384):
            if path == "graph":
                os.environ["FQSB_NO_SMALL"] = "1"
            try:
                q = fqsb.Line1d.System_Cuspy_Laplace(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / n,
                                                     dt=0.1, shape=[n], seed=0, distribution="weibull",
                                                     parameters=[2.0, 1.0, 1e-5], offset=-500.0, nchunk=1000)
            finally:
                os.environ.pop("FQSB_NO_SMALL", None)
            q.flowSteps(100, 1e-3)
            t0 = time.perf_counter()
            q.timeSteps(20000)
            t1 = time.perf_counter()
            q.u_frame = q.u_frame + 0.5
            i0 = q.inc
            t2 = time.perf_counter()
            q.minimise(max_iter=200000, max_iter_is_error=False)
            t3 = time.perf_counter()
            sizes[f"{path}_N{n}"] = {"time_steps_us_per_step": 1e6 * (t1 - t0) / 20000,
                                     "minimise_us_per_step": 1e6 * (t3 - t2) / max(1, q.inc - i0),
                                     "minimise_steps": q.inc - i0}
            del q
    out["sizes"] = sizes
    return out


def bench_line2d(fqsb, full=False):
    """Line2d System_Cuspy_Laplace on a 2048 x 2048 periodic grid: m = 1, eta = 0.2, mu = 1, k = 1,
    k_frame = 1/2048^2, dt = 0.1, Weibull(2,1)+1e-5 from pcg32 seed 2, 500 yield positions per site;
    cycles of eventDrivenStep(1e-5, kick=False), eventDrivenStep(1e-5, kick=True), minimise(tol=1e-5)
    (20 with --full, else 1 warm-up + 2 timed); flowSteps(200, v_frame = 1e-3) for the dynamics without
    the residual; then a regeneration sweep: u += 600 and back (every
    site crosses ~680 wells, so every chunk window is regenerated from its pcg32 stream, forward then
    backward)."""
    side = 2048
    n = side * side
    s = fqsb.Line2d.System_Cuspy_Laplace(m=1.0, eta=0.2, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1,
                                         shape=[side, side], seed=2, distribution="weibull",
                                         parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=500)
    ncycles = 20 if full else 2
    out = {"shape": [side, side], "cycles": ncycles, "per_cycle": []}
    if not full:
        s.eventDrivenStep(1e-5, False)
        s.eventDrivenStep(1e-5, True)
        s.minimise()
    tot_t, tot_steps = 0.0, 0
    for _ in range(ncycles):
        inc0 = s.inc
        t0 = time.perf_counter()
        s.eventDrivenStep(1e-5, False)
        s.eventDrivenStep(1e-5, True)
        t1 = time.perf_counter()
        ret = s.minimise()
        t2 = time.perf_counter()
        steps = s.inc - inc0
        tot_t += t2 - t0
        tot_steps += steps
        out["per_cycle"].append({"event_s": t1 - t0, "minimise_s": t2 - t1, "time_steps": steps, "ret": ret})
    ps = n * tot_steps / tot_t
    out.update(seconds=tot_t, time_steps=tot_steps, particle_steps_per_s=ps,
               hbm_frac_64B=BYTES_PER_PARTICLE_STEP * ps / 1e9 / peaks()[0])
    # dynamics without the residual: flowSteps(200) with the frame moving 1e-4 per step
    s.flowSteps(20, V_FRAME)
    t0 = time.perf_counter()
    s.flowSteps(200, V_FRAME)
    tf = time.perf_counter() - t0
    out["flow"] = {"steps": 200, "seconds": tf, "particle_steps_per_s": n * 200 / tf}
    u = s.u
    t0 = time.perf_counter()
    s.u = u + 600.0
    t1 = time.perf_counter()
    s.u = u
    t2 = time.perf_counter()
    out["regeneration_sweep"] = {"forward_s": t1 - t0, "backward_s": t2 - t1, "wells_crossed_per_site": "~680"}
    return out


def bench_batched(fqsb, full=False):
    """Batched form on all 4096 realisations of the size list (N_j log-uniform in [256, 65536] from
    pcg32 seed 3; pcg32 seed 1000+j; k_frame = 1/N_j; Weibull(2,1)+1e-5; 1000-position chunk, 64 kept),
    cycles of eventDrivenStep(1e-5, False), eventDrivenStep(1e-5, True), minimise(tol=1e-5) (50 with
    --full, else 1) with the tile shape the autotuner picks; against the plain path looped over a random
    sample of the realisations (256 with --full, else 64; seed 5) for the same cycles, scaled to all
    realisations by their share of the particles."""
    from frictionqpotspringblock_gb300 import autotune as A
    from frictionqpotspringblock_gb300 import batch as B

    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, distribution="weibull",
               parameters=[2.0, 1.0, 1e-5], offset=-100.0)
    sizes = B.log_uniform_sizes(4096, 256, 65536, seed=3)
    seeds = 1000 + np.arange(4096)
    ncycles = 50 if full else 1
    nloop = 256 if full else 64
    out = {"realisations": 4096, "particles": int(sizes.sum()), "cycles": ncycles}

    def make(sz, threads, ppt):
        return B.Line1d_System_Cuspy_Laplace(sz, 1000 + np.arange(len(sz)), 1.0 / sz, nchunk=1000, window=64,
                                             threads=threads, ppt=ppt, **par)

    t0 = time.perf_counter()
    threads, ppt = A.choose_tile(sizes[:512], make, use_cache=False)
    out.update(tile=[int(threads), int(ppt)], autotune_seconds=time.perf_counter() - t0)
    b = B.Line1d_System_Cuspy_Laplace(sizes, seeds, 1.0 / sizes, nchunk=1000, window=64, threads=threads, ppt=ppt,
                                      **par)
    t0 = time.perf_counter()
    r = b.quasistatic(ncycles, 1e-5)
    t = time.perf_counter() - t0
    ps = int((r["inc"][:, -1] * sizes).sum())
    steps = r["inc"][:, -1]
    out.update(seconds=t, particle_steps=ps, value=ps / t, converged=int(np.sum(r["status"] == 0)),
               steps_per_realisation={"mean": float(steps.mean()), "max": int(steps.max()),
                                      "min": int(steps.min())},
               # particle-steps done / (the longest realisation's steps x all particles): the share of the
               # launched tiles that had work, if every iteration launched every tile
               busy_fraction=ps / (float(steps.max()) * float(sizes.sum())))
    del b
    pick = np.sort(np.random.default_rng(5).choice(4096, nloop, replace=False))
    tp, pps = 0.0, 0
    for j in pick:
        s = fqsb.Line1d.System_Cuspy_Laplace(k_frame=1.0 / float(sizes[j]), shape=[int(sizes[j])], seed=int(seeds[j]),
                                             nchunk=1000, **par)
        t0 = time.perf_counter()
        for _ in range(ncycles):
            s.eventDrivenStep(1e-5, False)
            s.eventDrivenStep(1e-5, True)
            s.minimise()
        tp += time.perf_counter() - t0
        pps += s.inc * int(sizes[j])
        del s
    share = float(sizes[pick].sum()) / float(sizes.sum())
    out["plain_loop"] = {"sample": int(nloop), "sample_seed": 5, "seconds": tp, "particle_steps": pps,
                         "particle_share": share, "scaled_seconds": tp / share}
    out["speedup_vs_plain_loop"] = (tp / share) / t
    return out


def bench_adjoint(fqsb, full=False, N=65536, T=5000, K=100, last=500):
    """Adjoint of the differentiation workload: Line1d System_Smooth_Laplace, N = 65536, k_frame = 1/N,
    Weibull(2,1)+1e-5 seed 4, u_frame(t) = 1e-3 t + 0.05 sin(2 pi t / 500), T = 5000, checkpoints every
    100 steps, from u0 = the equilibrium at u_frame = 0 (minimise from u = v = 0) and v0 = 0;
    forward vs forward + backward wall time.  Gradient check: central
    finite differences (h = 1e-6) of the forward's loss along mu, k_interactions and eta, and along one
    random direction (seed 9, entries uniform in [0, 1)) of u0, v0 and the schedule each; relative error
    against the adjoint's directional derivative.  `fd_noise_rel` is the finite difference's own
    resolution relative to that derivative: 64 ulp of the loss (a sum of 500 x 65536 frame forces),
    divided by h."""
    s = fqsb.Line1d.System_Smooth_Laplace(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1,
                                          shape=[N], seed=4, distribution="weibull", parameters=[2.0, 1.0, 1e-5],
                                          offset=-100.0, nchunk=1000)
    t = np.arange(T)
    sched = 1e-3 * t + 0.05 * np.sin(2 * np.pi * t / 500)
    zero = np.zeros(N)
    params = np.array([1.0, 1.0, 0.1])
    s.minimise(max_iter=1000000)
    ueq = s.u

    def loss(u0=ueq, v0=zero, sc=sched, p=params):
        s.set_parameters(*p)
        s.u, s.v, s.a = u0, v0, zero
        return s.adjoint_forward(sc, K=K, last=last)

    for _ in range(2):
        loss()
    s.set_parameters(*params)
    s.u, s.v, s.a = ueq, zero, zero
    t0 = time.perf_counter()
    L0 = s.adjoint_forward(sched, K=K, last=last)
    tf = time.perf_counter() - t0
    t0 = time.perf_counter()
    gu, gv, gs, gp = s.adjoint_backward()
    tb = time.perf_counter() - t0
    out = {"particles": N, "steps": T, "checkpoint_every": K, "loss": L0, "forward_s": tf, "backward_s": tb,
           "backward_over_forward": tb / tf, "total_over_forward": (tf + tb) / tf}
    h = 1e-6
    noise = 64 * np.spacing(abs(L0)) / h
    checks = {}
    for i, name in enumerate(["mu", "k_interactions", "eta"]):
        e = np.zeros(3)
        e[i] = h
        fd = (loss(p=params + e) - loss(p=params - e)) / (2 * h)
        checks[name] = {"adjoint": float(gp[i]), "fd": fd, "rel_err": abs(fd - gp[i]) / abs(gp[i]),
                        "fd_noise_rel": noise / abs(gp[i])}
    rng = np.random.default_rng(9)
    for name, g, x in [("u0", gu, ueq), ("v0", gv, zero), ("schedule", gs, sched)]:
        d = rng.uniform(0.0, 1.0, x.shape)
        kw_p = {"u0": "u0", "v0": "v0", "schedule": "sc"}[name]
        fd = (loss(**{kw_p: x + h * d}) - loss(**{kw_p: x - h * d})) / (2 * h)
        an = float(np.dot(g.ravel(), d.ravel()))
        checks[name] = {"adjoint": an, "fd": fd, "rel_err": abs(fd - an) / abs(an), "fd_noise_rel": noise / abs(an)}
    out["gradient_check"] = checks
    return out


def bench_next_rows(fqsb, full=False, n=2 ** 22, side=2048, n_lr=16384, n_np=2 ** 17, steps=200):
    """The further interaction types, the no-passing minimiser and the thermal forcing, each on its own
    system (Cuspy, Weibull(2,1)+1e-5 seed 2, 200-position chunk, m = 1, eta = 0.1, mu = 1, dt = 0.1,
    k_frame = 1/N, u ~ N(0, 0.1^2)), timed with the handle's synchronous calls after 20 warm-up steps:
    flowSteps(steps, 1e-3) for Line1d Quartic (a1 = a2 = 1) and QuarticGradient (k2 = k4 = 1) at
    N = 2^22 and Line2d QuarticGradient at 2048 x 2048; flowSteps(steps // 5) for Line1d LongRange
    (alpha = 1, k = 1, all pairs) at N = 16384; the no-passing minimiser (Line1d Nopassing, N = 2^17)
    after a +0.5 frame jump, bounded at 5000 sweeps; Line1d Cuspy_Laplace_RandomForcing (mean 0,
    stddev 0.05, forcing seed 0, every particle redrawn every 100 increments, first at a uniform
    random increment in [0, 100)) at N = 2^22 (flowSteps(steps)) and at the reference example's
    N = 1000 (flowSteps(5000); examples/Line1d_System_Cuspy_Laplace_RandomForcing.py)."""
    par = dict(eta=0.1, mu=1.0, dt=0.1, seed=2, distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-100.0,
               nchunk=200)
    out = {}

    def flow(name, make, size, nsteps, extra=None):
        try:
            s = make()
            s.u = np.random.default_rng(2).normal(0.0, 0.1, size).reshape(s.shape)
            s.flowSteps(20, V_FRAME)
            t0 = time.perf_counter()
            s.flowSteps(nsteps, V_FRAME)
            dt = time.perf_counter() - t0
            r = {"particles": size, "steps": nsteps, "seconds": dt, "particle_steps_per_s": size * nsteps / dt}
            if extra:
                r.update(extra(size, nsteps, dt))
            out[name] = r
            del s
        except Exception as e:  # noqa: BLE001 -- the bench line must still be printed
            out[name] = {"error": f"{type(e).__name__}: {e}"}

    flow("Line1d_Cuspy_Quartic", lambda: fqsb.Line1d.System_Cuspy_Quartic(
        m=1.0, a1=1.0, a2=1.0, k_frame=1.0 / n, shape=[n], **par), n, steps)
    flow("Line1d_Cuspy_QuarticGradient", lambda: fqsb.Line1d.System_Cuspy_QuarticGradient(
        m=1.0, k2=1.0, k4=1.0, k_frame=1.0 / n, shape=[n], **par), n, steps)
    flow("Line2d_Cuspy_QuarticGradient", lambda: fqsb.Line2d.System_Cuspy_QuarticGradient(
        m=1.0, k2=1.0, k4=1.0, k_frame=1.0 / side ** 2, shape=[side, side], **par), side * side, steps)
    flow("Line1d_Cuspy_LongRange", lambda: fqsb.Line1d.System_Cuspy_LongRange(
        m=1.0, k_interactions=1.0, alpha=1.0, k_frame=1.0 / n_lr, shape=[n_lr], **par), n_lr, steps // 5,
        extra=lambda size, k, dt: {"pair_terms_per_s": size * (size - 1) * k / dt})

    def thermal(size):
        return fqsb.Line1d.System_Cuspy_Laplace_RandomForcing(
            m=1.0, k_interactions=1.0, k_frame=1.0 / size, mean=0.0, stddev=0.05, seed_forcing=0,
            dinc_init=np.random.default_rng(3).integers(0, 100, size), dinc=np.full(size, 100), shape=[size], **par)

    flow("Line1d_Cuspy_Laplace_RandomForcing", lambda: thermal(n), n, steps,
         extra=lambda size, k, dt: {"draws_per_s": size / 100 * k / dt})
    flow("Line1d_Cuspy_Laplace_RandomForcing_N1000", lambda: thermal(1000), 1000, 5000)
    try:
        s = fqsb.Line1d.System_Cuspy_Laplace_Nopassing(mu=1.0, k_interactions=1.0, k_frame=1.0 / n_np, shape=[n_np],
                                                       **{k: v for k, v in par.items() if k not in ("eta", "dt", "mu")})
        s.u_frame = 0.5
        t0 = time.perf_counter()
        ret = s.minimise(max_iter=5000, max_iter_is_error=False)
        dt = time.perf_counter() - t0
        out["Line1d_Cuspy_Laplace_Nopassing"] = {"particles": n_np, "seconds": dt, "converged": ret == 0,
                                                 "max_iter": 5000}
        del s
    except Exception as e:  # noqa: BLE001
        out["Line1d_Cuspy_Laplace_Nopassing"] = {"error": f"{type(e).__name__}: {e}"}
    return out


FORM_FUNCS = {"small_system": bench_small, "line2d": bench_line2d, "batched": bench_batched,
              "adjoint": bench_adjoint, "next_rows": bench_next_rows}


# ------------------------------------------------------------------------------------------ CPU arms

def cpu_baseline_sample(n_sample=2 ** 16, steps=3000, repeats=1):
    """Time the CPU oracle (loop-per-statement restatement of the reference, libm, sequential sums)
    on a bounded sample of the same workload: the first n_sample particles' parameters on a ring of
    n_sample, flowSteps(steps).  Returns particle-steps/s on one core."""
    from oracle import oracle as O

    s = O.line1d("Cuspy", shape=[n_sample], k_frame=1.0 / n_sample, **PAR, sum_mode=O.SUM_SEQUENTIAL,
                 math_mode=O.MATH_LIBM)
    s.u = np.random.default_rng(1).normal(0.0, 0.1, N_DEFAULT)[:n_sample]
    s.flowSteps(20, V_FRAME)
    t0 = time.perf_counter()
    for _ in range(repeats):
        s.flowSteps(steps, V_FRAME)
    dt = time.perf_counter() - t0
    return n_sample * steps * repeats / dt, dt


def _mem_available_bytes():
    try:
        for line in pathlib.Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def run_reference(args, rank, world):
    """CPU reference arm on the GPU arm's workload: the reference's time-integration path restated in C
    (the reference's own build needs prrng / xtensor / GooseFEM, absent here) and built with OpenMP, so
    its per-particle loops run over all host cores (flowSteps has no reductions: the results equal the
    single-threaded build's).  Same N = 2^22 ring, parameters, seeds and initial state as the GPU arm;
    each bench step is flowSteps(k) with k sized so that the warm-up and timed steps take about two
    minutes (the GPU arm's step is flowSteps(1000)); the metric is the same particle-steps/s."""
    if rank != 0:
        return
    from oracle import oracle as O

    N = args.n
    nchunk = args.nchunk
    need = N * nchunk * 8 + 16 * N * 8
    avail = _mem_available_bytes()
    note = ""
    if avail is not None and need > 0.8 * avail:
        nchunk = max(34, int((0.8 * avail - 16 * N * 8) / (8 * N)))
        note = (f"; {nchunk} instead of {args.nchunk} yield positions per particle held in host memory "
                f"(the yield sequence and the trajectory do not depend on it)")
    O.build(threads=True)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    s = O.line1d("Cuspy", shape=[N], k_frame=1.0 / N, **dict(PAR, nchunk=nchunk), sum_mode=O.SUM_SEQUENTIAL,
                 math_mode=O.MATH_LIBM, threads=True)
    s.u = np.random.default_rng(1).normal(0.0, 0.1, N)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    s.flowSteps(10, V_FRAME)
    rate = N * 10 / (time.perf_counter() - t0)
    budget = 120.0 / (args.steps + args.warmup)
    inner = int(min(INNER, max(10, round(budget * rate / N))))
    for _ in range(args.warmup):
        s.flowSteps(inner, V_FRAME)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s.flowSteps(inner, V_FRAME)
        times.append(time.perf_counter() - t0)
    total_time = sum(times)
    value = N * inner * args.steps / total_time
    sample = (f"the full N={N} ring of the GPU arm's workload (same parameters, seeds and u0), each bench step "
              f"flowSteps({inner}) instead of flowSteps({INNER}); the reference's path restated in C (oracle/), "
              f"built -O2 -ffp-contract=off -fopenmp, {cores} threads over the per-particle loops; construction "
              f"{t_build:.1f} s (untimed){note}")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total_time / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload(N), "particles": N, "time_steps_per_step": inner,
                   "l2": "inputs larger than L2 on the GPU arm"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------ main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--nchunk", type=int, default=2000, help="yield positions per particle (profiling cases only)")
    ap.add_argument("--no-minimise", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip every entry of `forms`")
    ap.add_argument("--forms", default=",".join(FORMS), help=f"comma-separated subset of {','.join(FORMS)}")
    ap.add_argument("--full", action="store_true", help="run the forms' protocols at their configured sizes")
    ap.add_argument("--only-forms", action="store_true", help="skip the main workload; run the selected forms")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)

    import frictionqpotspringblock_gb300 as fqsb
    from frictionqpotspringblock_gb300 import _capi

    forms_sel = [] if args.no_forms else [f for f in args.forms.split(",") if f]
    if args.only_forms:
        forms = {f: _guard(FORM_FUNCS[f], fqsb, full=args.full) for f in forms_sel}
        if rank == 0:
            print(json.dumps({"forms": forms, "full": args.full}), flush=True)
        return

    N = args.n
    par = dict(PAR)
    par["nchunk"] = args.nchunk
    system = fqsb.Line1d.System_Cuspy_Laplace(k_frame=1.0 / N, shape=[N], device=local_rank, **par)
    u0 = np.random.default_rng(1).normal(0.0, 0.1, N)
    system.u = u0
    stream = torch.cuda.ExternalStream(system.stream)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    for _ in range(args.warmup):
        system.flowSteps(INNER, V_FRAME)

    # ---- device-resident timed region
    clocks = ClockSampler(local_rank)
    barrier()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_wall0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        system.flowSteps(INNER, V_FRAME)
    e1.record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    dev_s = max_over_ranks(e0.elapsed_time(e1) / 1e3)
    launches = args.steps * INNER
    particle_steps = N * INNER * args.steps
    value = world * particle_steps / dev_s
    kernel_s = dev_s / launches
    hbm_peak, peak_kind = peaks()
    achieved_gbs = BYTES_PER_PARTICLE_STEP * N / kernel_s / 1e9

    # ---- end-to-end through the public API with host buffers
    host_u = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_v = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    host_u[:] = system.u
    host_v[:] = system.v
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        system.u = host_u
        system.v = host_v
        system.flowSteps(INNER, V_FRAME)
        out = system.u
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * particle_steps / e2e_s
    del out

    # ---- the frame jump and minimise of the configuration (timed once)
    minimise = None
    if not args.no_minimise:
        system.u_frame = system.u_frame + 0.5
        barrier()
        t0 = time.perf_counter()
        inc0 = system.inc
        ret = system.minimise(tol=1e-5)
        barrier()
        ms = time.perf_counter() - t0
        steps = system.inc - inc0
        minimise = {"seconds": ms, "steps": steps, "ret": ret, "us_per_step": 1e6 * ms / max(1, steps),
                    "over_flow_step": (ms / max(1, steps)) / kernel_s}
    del system

    # ---- arithmetic peaks of this GPU (the fp64 roofline's denominator), measured here
    fp64_peak = _guard(_capi.measure_arith, "add", 0, local_rank)
    fp64_peak_mul = _guard(_capi.measure_arith, "mul", 0, local_rank)

    forms = {f: _guard(FORM_FUNCS[f], fqsb, full=args.full) for f in forms_sel}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline:
        v, secs = cpu_baseline_sample()
        cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"oracle (reference restated in C, loop per statement, libm, sequential sums), "
                         f"N=65536 ring of the same parameters, flowSteps(3000), {secs:.1f} s on 1 core"}
    figs = profile_figures()
    traffic = figs["traffic_bytes_per_launch"] / figs["traffic_particles"] * N
    fp64_gops = FP64_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9
    fp64_pipe_gops = FP64_PIPE_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9
    peak_gops = fp64_peak if isinstance(fp64_peak, float) else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload(N), "particles": N, "time_steps_per_step": INNER,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (state + well cache ~270 MB vs 129 MB L2), no flush"},
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": 2 * 8 * N,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu capture of " + STEP_PROFILE.name + ", scaled by N)",
                     "peak_kind": peak_kind, "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
                     "kernel": "k_step_line<Cuspy, Laplace1d, 2 per thread>", "kernel_us": kernel_s * 1e6},
        "fp64": {"ops_per_particle_step": FP64_OPS_PER_PARTICLE_STEP,
                 "ops_on_fp64_pipe": FP64_PIPE_OPS_PER_PARTICLE_STEP,
                 "ops_on_integer_pipes": FP64_OPS_PER_PARTICLE_STEP - FP64_PIPE_OPS_PER_PARTICLE_STEP,
                 "achieved_gops": fp64_gops, "fp64_pipe_gops": fp64_pipe_gops,
                 "peak_gops": fp64_peak, "peak_mul_gops": fp64_peak_mul,
                 "peak_source": "fqsb_measure_arith in this run (8 independent DADD chains per thread)",
                 "frac": fp64_gops / peak_gops if peak_gops else None,
                 "frac_fp64_pipe": fp64_pipe_gops / peak_gops if peak_gops else None},
        "clocks": clk,
        "wall_s": t_wall,
        "minimise": minimise,
        "forms": forms,
        "forms_full": args.full,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
