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
run once and their wall time is reported (minimise_s).

`value` times the device-resident steps (state already in HBM); `e2e` times
the same steps through the public API with host buffers: each step copies u
and v from pinned host memory into the system, runs flowSteps(1000) and reads
u back.  `--impl reference` times the CPU reference path instead (the CPU
oracle, a loop-per-statement restatement of the reference, on the host
cores), on bounded samples of the same workload.

Multi-GPU (torchrun): the plain path does not shard (one system fits one GPU),
so every rank runs an independent replica (weak scaling); value = sum of the
ranks' particle-steps / max rank time.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
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
# DRAM bytes per particle per step of the step kernel from one ncu capture (N = 2^21, dram__bytes_read.sum
# + dram__bytes_write.sum = 147.49 MB per launch; profiles/k_step_line_cuspy_laplace1d_N4M.md), scaled by N
TRAFFIC_BYTES_PER_PARTICLE_STEP = 147.49e6 / 2097152
FP64_OPS_PER_PARTICLE_STEP = 24  # binary64 add/mul of the exact-order step; compares and 2^k scalings are integer work
# of those, the step kernel issues these on the fp64 pipe; the rest (the 8 multiplications and the 2 additions of
# the position update) run bit-identically on the integer pipes (csrc/fq_soft64.h)
FP64_PIPE_OPS_PER_PARTICLE_STEP = 14


def workload(n):
    return (f"Line1d System_Cuspy_Laplace N={n} ring, m=1 eta=0.1 mu=1 k=1 k_frame=1/N dt=0.1, "
            f"weibull(2,1)+1e-5 nchunk=2000 seed=1, u0~N(0,0.1^2); step = flowSteps({INNER}, v_frame=1e-3) "
            f"(u_frame +1e-4 per time step); then u_frame += 0.5 and minimise(tol=1e-5)")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


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


def bench_batched(fqsb, n_inst=512, n_loop=32):
    """Batched form on the first n_inst realisations of the 4096-realisation size list (log-uniform in
    [256, 65536] from pcg32 seed 3; seed 1000+j; k_frame = 1/N_j; Weibull(2,1)+1e-5; 1000-position
    chunk), one quasistatic cycle each, with the tile shape the autotuner picks; against looping the
    plain path over the first n_loop."""
    from frictionqpotspringblock_gb300 import autotune as A
    from frictionqpotspringblock_gb300 import batch as B

    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, dt=0.1, distribution="weibull",
               parameters=[2.0, 1.0, 1e-5], offset=-100.0)
    sizes = B.log_uniform_sizes(4096, 256, 65536, seed=3)
    seeds = 1000 + np.arange(4096)
    out = {}

    # tile shape (threads x particles per thread) from the autotuner: timed on a sample of the batch
    def make(sz, threads, ppt):
        return B.Line1d_System_Cuspy_Laplace(sz, 1000 + np.arange(len(sz)), 1.0 / sz, nchunk=1000, window=64,
                                             threads=threads, ppt=ppt, **par)

    t0 = time.perf_counter()
    threads, ppt = A.choose_tile(sizes[:n_inst], make, use_cache=False)
    out.update(tile=[int(threads), int(ppt)], autotune_seconds=time.perf_counter() - t0)
    b = B.Line1d_System_Cuspy_Laplace(sizes[:n_inst], seeds[:n_inst], 1.0 / sizes[:n_inst], nchunk=1000, window=64,
                                      threads=threads, ppt=ppt, **par)
    t0 = time.perf_counter()
    r = b.quasistatic(1, 1e-5)
    t = time.perf_counter() - t0
    ps = int((r["inc"][:, -1] * sizes[:n_inst]).sum())
    out.update(realisations=n_inst, particles=int(sizes[:n_inst].sum()), seconds=t, particle_steps=ps, value=ps / t)
    del b
    b = B.Line1d_System_Cuspy_Laplace(sizes[:n_loop], seeds[:n_loop], 1.0 / sizes[:n_loop], nchunk=1000, window=64,
                                      threads=threads, ppt=ppt, **par)
    t0 = time.perf_counter()
    r = b.quasistatic(1, 1e-5)
    tb = time.perf_counter() - t0
    del b
    tp = 0.0
    for j in range(n_loop):
        s = fqsb.Line1d.System_Cuspy_Laplace(k_frame=1.0 / float(sizes[j]), shape=[int(sizes[j])], seed=int(seeds[j]),
                                             nchunk=1000, **par)
        t0 = time.perf_counter()
        s.eventDrivenStep(1e-5, False)
        s.eventDrivenStep(1e-5, True)
        s.minimise()
        tp += time.perf_counter() - t0
        del s
    out.update(loop_realisations=n_loop, loop_plain_seconds=tp, loop_batched_seconds=tb, speedup_vs_plain_loop=tp / tb)
    return out


def bench_adjoint(fqsb, N=65536, T=5000, K=100, last=500):
    """Adjoint of the differentiation workload: Line1d System_Smooth_Laplace, N = 65536, k_frame = 1/N,
    Weibull(2,1)+1e-5 seed 4, u0 = v0 = 0, u_frame(t) = 1e-3 t + 0.05 sin(2 pi t / 500), T = 5000,
    checkpoints every 100 steps; forward vs forward + backward wall time."""
    s = fqsb.Line1d.System_Smooth_Laplace(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1,
                                          shape=[N], seed=4, distribution="weibull", parameters=[2.0, 1.0, 1e-5],
                                          offset=-100.0, nchunk=1000)
    t = np.arange(T)
    sched = 1e-3 * t + 0.05 * np.sin(2 * np.pi * t / 500)
    zero = np.zeros(N)
    for _ in range(2):
        s.u, s.v, s.a = zero, zero, zero
        s.adjoint_forward(sched, K=K, last=last)
    s.u, s.v, s.a = zero, zero, zero
    t0 = time.perf_counter()
    loss = s.adjoint_forward(sched, K=K, last=last)
    tf = time.perf_counter() - t0
    t0 = time.perf_counter()
    gu, gv, gs, gp = s.adjoint_backward()
    tb = time.perf_counter() - t0
    return {"particles": N, "steps": T, "checkpoint_every": K, "loss": loss, "forward_s": tf, "backward_s": tb,
            "backward_over_forward": tb / tf, "total_over_forward": (tf + tb) / tf,
            "grad_norms": {"u0": float(np.linalg.norm(gu)), "schedule": float(np.linalg.norm(gs)),
                           "params": [float(x) for x in gp]}}


def bench_small(fqsb, cycles=20, cpu_cycles=3):
    """Small system: Line1d System_Cuspy_Laplace N = 1024, k_frame = 1/1024, Weibull(2,1)+1e-5 seed 0,
    1000-position chunk shifted per particle so that u = 0 is the centre of well 500; cycles of
    eventDrivenStep(1e-5, kick=False), eventDrivenStep(1e-5, kick=True), minimise(tol=1e-5)."""
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / 1024, dt=0.1, shape=[1024], seed=0,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], nchunk=1000)
    raw = fqsb.Line1d.System_Cuspy_Laplace(offset=0.0, **par).chunk.data
    offp = -0.5 * (raw[:, 500] + raw[:, 501])
    s = fqsb.Line1d.System_Cuspy_Laplace(offset=0.0, offset_per_particle=offp, **par)
    s.eventDrivenStep(1e-5, False)
    s.eventDrivenStep(1e-5, True)
    s.minimise(max_iter=1000000)
    inc0 = s.inc
    t0 = time.perf_counter()
    for _ in range(cycles):
        s.eventDrivenStep(1e-5, False)
        s.eventDrivenStep(1e-5, True)
        s.minimise(max_iter=1000000)
    t = time.perf_counter() - t0
    out = {"particles": 1024, "cycles": cycles, "seconds_per_cycle": t / cycles,
           "steps_per_cycle": (s.inc - inc0) / cycles, "us_per_step": 1e6 * t / max(1, s.inc - inc0)}
    if cpu_cycles > 0:
        # the same protocol on the CPU oracle (the reference restated: libm, sequential sums), one core
        from oracle import oracle as O

        r = O.line1d("Cuspy", offset=0.0, offset_per_particle=offp, sum_mode=O.SUM_SEQUENTIAL, math_mode=O.MATH_LIBM,
                     **par)
        r.eventDrivenStep(1e-5, False)
        r.eventDrivenStep(1e-5, True)
        r.minimise(max_iter=1000000)
        inc0 = r.inc
        t0 = time.perf_counter()
        for _ in range(cpu_cycles):
            r.eventDrivenStep(1e-5, False)
            r.eventDrivenStep(1e-5, True)
            r.minimise(max_iter=1000000)
        tc = time.perf_counter() - t0
        out["cpu_oracle"] = {"cycles": cpu_cycles, "cores": 1, "us_per_step": 1e6 * tc / max(1, r.inc - inc0)}
        out["speedup_vs_cpu_oracle"] = out["cpu_oracle"]["us_per_step"] / out["us_per_step"]
    return out


def bench_next_rows(fqsb, n=2 ** 22, side=2048, n_lr=16384, n_np=2 ** 17, steps=200):
    """The further interaction types and the no-passing minimiser, each on its own system (Cuspy,
    Weibull(2,1)+1e-5 seed 2, 200-position chunk, m = 1, eta = 0.1, mu = 1, dt = 0.1, k_frame = 1/N,
    u ~ N(0, 0.1^2)), timed with the handle's synchronous calls after 20 warm-up steps:
    flowSteps(steps, 1e-3) for Line1d Quartic (a1 = a2 = 1) and QuarticGradient (k2 = k4 = 1) at
    N = 2^22 and Line2d QuarticGradient at 2048 x 2048; flowSteps(steps // 5) for Line1d LongRange
    (alpha = 1, k = 1, all pairs) at N = 16384; the no-passing minimiser (Line1d Nopassing, N = 2^17)
    after a +0.5 frame jump, bounded at 5000 sweeps.  A failure is recorded, not raised."""
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


def _ref_worker(args):
    n_sample, steps, nsteps_total, warm = args
    from oracle import oracle as O

    s = O.line1d("Cuspy", shape=[n_sample], k_frame=1.0 / n_sample, **PAR, sum_mode=O.SUM_SEQUENTIAL,
                 math_mode=O.MATH_LIBM)
    s.u = np.random.default_rng(1).normal(0.0, 0.1, n_sample)
    for _ in range(warm):
        s.flowSteps(steps, V_FRAME)
    times = []
    for _ in range(nsteps_total):
        t0 = time.perf_counter()
        s.flowSteps(steps, V_FRAME)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, rank, world):
    """CPU reference arm: the reference path restated on the host (the reference's own build needs
    prrng / xtensor / GooseFEM, absent here), one independent sample system per host core."""
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle import oracle as O

    O.build()
    cores = os.cpu_count() or 1
    n_sample, steps = 2 ** 14, 200
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_ref_worker, [(n_sample, steps, args.steps, args.warmup)] * cores)
    per_step = [max(r[i] for r in res) for i in range(args.steps)]
    total_time = sum(per_step)
    value = cores * n_sample * steps * args.steps / total_time
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
        "config": {"workload": workload(args.n), "l2": "inputs larger than L2 on the GPU arm"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} independent systems of N={n_sample} (one per core), "
                                   f"each step flowSteps({steps}); the reference's path restated in C "
                                   "(oracle/), built -O2 -ffp-contract=off"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    ap.add_argument("--no-forms", action="store_true", help="skip the batched / adjoint / small-system extras")
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
        minimise = {"seconds": time.perf_counter() - t0, "steps": system.inc - inc0, "ret": ret}

    forms = {}
    if not args.no_forms:
        forms["batched"] = bench_batched(fqsb)
        forms["adjoint"] = bench_adjoint(fqsb)
        forms["small_system"] = bench_small(fqsb)
        forms["next_rows"] = bench_next_rows(fqsb)

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        v, secs = cpu_baseline_sample()
        cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"oracle (reference restated in C, loop per statement, libm, sequential sums), "
                         f"N=65536 ring of the same parameters, flowSteps(3000), {secs:.1f} s on 1 core"}
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
                     "frac": achieved_gbs / hbm_peak, "traffic": TRAFFIC_BYTES_PER_PARTICLE_STEP * N,
                     "traffic_unit": "bytes per launch (ncu capture at N=2^21 scaled by N)", "peak_kind": peak_kind,
                     "algorithmic_bytes_per_particle_step": BYTES_PER_PARTICLE_STEP,
                     "kernel": "k_step_line<Cuspy, Laplace1d, units, 2 per thread>",
                     "kernel_us": kernel_s * 1e6},
        "fp64": {"ops_per_particle_step": FP64_OPS_PER_PARTICLE_STEP,
                 "ops_on_fp64_pipe": FP64_PIPE_OPS_PER_PARTICLE_STEP,
                 "ops_on_integer_pipes": FP64_OPS_PER_PARTICLE_STEP - FP64_PIPE_OPS_PER_PARTICLE_STEP,
                 "achieved_gops": FP64_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9,
                 "fp64_pipe_gops": FP64_PIPE_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9,
                 "peak_gops": 505.0, "peak_source": "profiles/fp64_throughput_gb300.md",
                 "frac": FP64_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9 / 505.0,
                 "frac_fp64_pipe": FP64_PIPE_OPS_PER_PARTICLE_STEP * N / kernel_s / 1e9 / 505.0},
        "clocks": clk,
        "wall_s": t_wall,
        "minimise": minimise,
        "forms": forms,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
