"""The CUDA path against the reference's own arithmetic, on the benchmark configurations.

The other GPU parity tests compare with the oracle in its portable mode (the device's elementary
functions and pairwise sums), bit for bit.  Here the oracle runs as the reference computes: glibc's
log / pow / sin (prrng's Weibull transform scale * pow(-log(1 - r), 1 / k) + offset, the Smooth
potential's sin, detail.h:379-409) and sequential sums (xtensor's norm_l2 / mean).  glibc's log and
pow are not correctly rounded, so about 0.1% of the Weibull yield distances differ from the device's
in the last bit; the two runs then follow trajectories that differ by rounding only.

The bar (the plain path's correctness requirement): identical well indices after every minimise and
at every check of a dynamic run, identical step counts, and u / v / f within 1e-12 relative per
step.  "Relative" is taken against the scale of the quantity's terms, stated per test: positions
against max |u|; forces and accelerations, which are sums of terms, against the largest term (or,
after a quasistatic cycle, against max |u|, the positions they are differences of); velocities
against max |v|.  Over many steps rounding differences are carried along (and, in the Smooth
potential's unstable regions, amplified), so long dynamic runs are held to that bar per step -- one
step from the reference's state -- and to identical well indices throughout; the accumulated drift
is asserted more loosely (stated per test) and printed.
"""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fqsb = pytest.importorskip("frictionqpotspringblock_gb300")

RTOL = 1e-12
FORCES = ["f", "f_potential", "f_interactions", "f_frame", "f_damping"]


def rel(g, r, scale):
    return float(np.max(np.abs(np.asarray(g) - np.asarray(r)))) / scale


@pytest.mark.timeout(900)
def test_small_system_protocol():
    """Line1d System_Cuspy_Laplace, N = 1024, m = 1, eta = 0.1, mu = 1, k = 1, k_frame = 1/1024,
    dt = 0.1, Weibull(2,1)+1e-5 from pcg32 seed 0, 1000 yield positions per particle shifted per
    particle so that u = 0 is the centre of well 500; u = v = 0, u_frame = 0; 100 cycles of
    eventDrivenStep(1e-5, kick=False), eventDrivenStep(1e-5, kick=True), minimise(tol=1e-5,
    max_iter=1e6) (examples/Line1d_Cuspy_Laplace.py:41-60).  Every cycle: well indices and increment
    identical; u and the forces within 1e-12 of max |u|; u_frame within 1e-11 relative, and the
    returned frame displacements within the same 1e-11 of |u_frame| (each event moves the frame by
    du (k_frame + mu) / k_frame, which amplifies a last-bit difference of a yield position 1025
    times); the recorded mean frame force within 1e-11 of k_frame |u_frame| (the magnitude of the
    terms it is formed from, and the frame position's tolerance)."""
    N = 1024
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1, shape=[N], seed=0,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], nchunk=1000)
    # yield positions 500 and 501 of every particle without shift; the chunk window of that system was
    # moved so that u = 0 (below its first yield position) sits inside it, so columns are offset by start
    plain = O.line1d("Cuspy", offset=0.0, sum_mode=O.SUM_SEQUENTIAL, math_mode=O.MATH_LIBM, **par)
    raw, start = plain.chunk.data, plain.chunk.start
    rows = np.arange(N)
    offp = -0.5 * (raw[rows, 500 - start] + raw[rows, 501 - start])
    ref = O.line1d("Cuspy", offset=0.0, offset_per_particle=offp, sum_mode=O.SUM_SEQUENTIAL,
                   math_mode=O.MATH_LIBM, **par)
    gpu = fqsb.Line1d.System_Cuspy_Laplace(offset=0.0, offset_per_particle=offp, **par)
    assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align)
    assert np.all(gpu.chunk.index_at_align == 500)
    ydiff = int(np.sum(gpu.chunk.data != ref.chunk.data))
    worst = {"u": 0.0, "f": 0.0, "u_frame": 0.0, "f_frame_mean": 0.0}
    for cycle in range(100):
        for kick in (False, True):
            a = gpu.eventDrivenStep(1e-5, kick)
            b = ref.eventDrivenStep(1e-5, kick)
            # the frame displacement: a difference of frame positions, held to their tolerance
            assert abs(a - b) <= 10 * RTOL * max(abs(ref.u_frame), 1.0), (cycle, kick, a, b)
        assert gpu.minimise(max_iter=1000000) == ref.minimise(max_iter=1000000) == 0
        assert gpu.inc == ref.inc, cycle
        assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align), cycle
        scale = float(np.max(np.abs(ref.u)))
        worst["u"] = max(worst["u"], rel(gpu.u, ref.u, scale))
        worst["f"] = max(worst["f"], max(rel(getattr(gpu, k), getattr(ref, k), scale) for k in FORCES))
        assert worst["u"] <= RTOL and worst["f"] <= RTOL, (cycle, worst)
        assert np.array_equal(gpu.v, ref.v)  # both quenched
        d_uf = abs(gpu.u_frame - ref.u_frame) / abs(ref.u_frame)
        d_ff = abs(np.mean(gpu.f_frame) - np.mean(ref.f_frame)) / (par["k_frame"] * abs(ref.u_frame))
        worst["u_frame"] = max(worst["u_frame"], d_uf)
        worst["f_frame_mean"] = max(worst["f_frame_mean"], d_ff)
        assert d_uf <= 10 * RTOL and d_ff <= 10 * RTOL, (cycle, d_uf, d_ff)
    print(f"\nsmall-system protocol: {ydiff} of {gpu.chunk.data.size} yield positions differ in the last bits; "
          f"worst relative differences over 100 cycles: {worst}")


def c5_pair(pot, n):
    kw = dict(kappa=1.0) if pot == "SemiSmooth" else {}
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1, shape=[n], seed=4,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=1000, **kw)
    gpu = getattr(fqsb.Line1d, f"System_{pot}_Laplace")(**par)
    ref = O.line1d(pot, sum_mode=O.SUM_SEQUENTIAL, math_mode=O.MATH_LIBM, **par)
    return gpu, ref


@pytest.mark.timeout(900)
@pytest.mark.parametrize("pot", ["Smooth", "SemiSmooth"])
def test_weibull_dynamics(pot):
    """Line1d System_{Smooth,SemiSmooth}_Laplace (kappa = 1), N = 65536, k_frame = 1/N, Weibull(2,1)+1e-5
    from pcg32 seed 4, u = v = 0, 1000 steps with u_frame(t) = 1e-3 t + 0.05 sin(2 pi t / 500) set before
    step t (the differentiation workload's forward).  Both run independently; every 100 steps the well
    indices must be identical and u within 1e-11 of max |u| (accumulated drift).  At the same points one
    step is taken from the reference's state by a second pair of systems, which must agree within 1e-12
    relative: u against max |u|, v against max |v|, and a and the forces against the largest force term
    max(|f_potential|, |f_interactions|) they are summed from."""
    N = 65536
    gpu, ref = c5_pair(pot, N)
    probe, probe_ref = c5_pair(pot, N)  # one step from the reference's state
    T = 1000
    t = np.arange(T + 1)
    sched = 1e-3 * t + 0.05 * np.sin(2 * np.pi * t / 500)
    drift, step_err = 0.0, 0.0
    for k in range(T):
        gpu.u_frame = sched[k]
        ref.u_frame = sched[k]
        gpu.timeStep()
        ref.timeStep()
        if k % 100 != 99:
            continue
        assert np.array_equal(gpu.chunk.index_at_align, ref.chunk.index_at_align), k
        drift = max(drift, rel(gpu.u, ref.u, float(np.max(np.abs(ref.u)))))
        assert drift <= 10 * RTOL, (k, drift)
        state = (ref.u, ref.v, ref.a)
        for s in (probe, probe_ref):
            s.u_frame = sched[k + 1]
            s.u, s.v, s.a = state
            s.timeStep()
        assert np.array_equal(probe.chunk.index_at_align, probe_ref.chunk.index_at_align), k
        fscale = max(float(np.max(np.abs(probe_ref.f_potential))), float(np.max(np.abs(probe_ref.f_interactions))))
        errs = {"u": rel(probe.u, probe_ref.u, float(np.max(np.abs(probe_ref.u)))),
                "v": rel(probe.v, probe_ref.v, float(np.max(np.abs(probe_ref.v)))),
                "a": rel(probe.a, probe_ref.a, fscale)}
        errs.update({name: rel(getattr(probe, name), getattr(probe_ref, name), fscale) for name in FORCES})
        step_err = max(step_err, max(errs.values()))
        assert all(e <= RTOL for e in errs.values()), (k, errs)
    print(f"\n{pot}: worst one-step difference {step_err:.2e} (relative), accumulated u drift {drift:.2e} "
          f"of max |u| after {T} steps")
