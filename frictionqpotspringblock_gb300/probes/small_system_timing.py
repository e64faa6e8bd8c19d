"""Time steps of small Line1d Cuspy systems: timeSteps(20000), then a +0.5 frame jump and minimise.

Prints microseconds per time step for each N.  Line1d System_Cuspy_Laplace, m = 1, eta = 0.1,
mu = 1, k = 1, k_frame = 1/N, dt = 0.1, Weibull(2,1)+1e-5 seed 0, offset -500, nchunk 1000.
Set FQSB_NO_SMALL=1 to time the CUDA-graph path instead of the one-cluster kernel.
Run from the repository root:  python frictionqpotspringblock_gb300/probes/small_system_timing.py 64,1024
"""

import os
import pathlib
import sys
import time

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parents[2]))

import frictionqpotspringblock_gb300 as fqsb  # noqa: E402


def make(n):
    return fqsb.Line1d.System_Cuspy_Laplace(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1,
                                            shape=[n], seed=0, distribution="weibull", parameters=[2.0, 1.0, 1e-5],
                                            offset=-500.0, nchunk=1000)


def main():
    sizes = [int(x) for x in (sys.argv[1] if len(sys.argv) > 1 else "64,1024,4096,8192").split(",")]
    for n in sizes:
        s = make(n)
        s.flowSteps(100, 1e-3)
        k = 20000
        t0 = time.perf_counter()
        s.timeSteps(k)
        t1 = time.perf_counter()
        s.u_frame = s.u_frame + 0.5
        i0 = s.inc
        t2 = time.perf_counter()
        s.minimise(max_iter=200000, max_iter_is_error=False)
        t3 = time.perf_counter()
        path = "graph" if os.environ.get("FQSB_NO_SMALL") == "1" else "cluster"
        print(f"N={n} path={path} timeSteps {1e6 * (t1 - t0) / k:.2f} us/step; "
              f"minimise {1e6 * (t3 - t2) / max(1, s.inc - i0):.2f} us/step ({s.inc - i0} steps)", flush=True)


if __name__ == "__main__":
    main()
