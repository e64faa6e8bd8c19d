"""The adjoint against torch autograd through an unrolled FP64 step and against finite differences.

The reference has no derivatives; the forward being differentiated is its timeStep with u_frame
set before every step (detail.h:1539-1570).  The torch reference below restates that step with
torch float64 operations (wells held at the forward's, read from the system), so torch autograd
gives an independent gradient.  Tolerances: 1e-9 relative against torch (same FP64 maths, different
summation order and sin/cos rounding), 1e-6 relative against central finite differences (h = 1e-6),
the gradient-error requirement of the differentiation workload.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
fqsb = pytest.importorskip("frictionqpotspringblock_gb300")
from frictionqpotspringblock_gb300.autograd import trajectory_loss  # noqa: E402

N, T, K, LAST = 96, 130, 50, 40


def make(kind):
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=0.05, dt=0.1, shape=[N], seed=4,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-30.0, nchunk=200)
    if kind == "Smooth":
        return fqsb.Line1d.System_Smooth_Laplace(**par)
    if kind == "SemiSmooth":
        return fqsb.Line1d.System_SemiSmooth_Laplace(kappa=0.7, **par)
    return fqsb.Line1d.System_Cuspy_Laplace(**par)


def inputs(seed=0):
    rng = np.random.default_rng(seed)
    u0 = rng.normal(0.0, 0.05, N)
    v0 = rng.normal(0.0, 0.01, N)
    t = np.arange(T)
    sched = 1e-3 * t + 0.05 * np.sin(2 * np.pi * t / 50)
    params = np.array([0.9, 1.1, 0.12])
    return u0, v0, sched, params


def torch_loss(kind, system, u0, v0, sched, params, kappa=0.7):
    """Unrolled FP64 forward in torch with the forward's wells (left, right yield per particle)."""
    yl = torch.tensor(system.chunk.left_of_align, dtype=torch.float64)
    yr = torch.tensor(system.chunk.right_of_align, dtype=torch.float64)
    mu, k, eta = params[0], params[1], params[2]
    m, dt, kf = 1.0, 0.1, 0.05
    u, v, a = u0, v0, torch.zeros_like(u0)
    acc = 0.0
    for t in range(T):
        up = (u + dt * v) + ((0.5 * dt) * dt) * a
        if kind == "Smooth":
            umin = 0.5 * (yl + yr)
            dy = 0.5 * (yr - yl)
            fp = -mu * dy / math.pi * torch.sin(math.pi * (up - umin) / dy)
        elif kind == "SemiSmooth":
            xi = 0.5 * (yl + yr)
            u_r = (mu * xi + kappa * yr) / (mu + kappa)
            u_l = (mu * xi + kappa * yl) / (mu + kappa)
            fp = torch.where(up < u_l, kappa * (up - yl),
                             torch.where(up <= u_r, mu * (0.5 * (yl + yr) - up), kappa * (up - yr)))
        else:
            fp = mu * (0.5 * (yl + yr) - up)
        fi = k * ((torch.roll(up, 1) - 2 * up) + torch.roll(up, -1))
        ff = kf * (sched[t] - up)
        s = (ff + fp) + fi
        v1 = v + dt * a
        a1 = (s + (-eta) * v1) / m
        v2 = v + (0.5 * dt) * (a + a1)
        a2 = (s + (-eta) * v2) / m
        v3 = v + (0.5 * dt) * (a + a2)
        a3 = (s + (-eta) * v3) / m
        if t >= T - LAST:
            acc = acc + torch.mean(ff)
        u, v, a = up, v3, a3
    return acc / LAST + 0.5 * torch.mean(u * u)


@pytest.mark.parametrize("kind", ["Smooth", "SemiSmooth", "Cuspy"])
def test_adjoint_matches_torch_autograd(kind):
    system = make(kind)
    u0, v0, sched, params = inputs()
    # start from a minimised equilibrium with a small perturbation, so that no particle changes well
    # and the torch restatement (which holds the wells) follows the same trajectory
    system.set_parameters(*params)
    system.minimise()
    left, right = system.chunk.left_of_align, system.chunk.right_of_align
    u0 = system.u + 1e-3 * (right - left) * np.random.default_rng(3).uniform(-1, 1, N)
    v0 = 1e-2 * v0
    sched = 1e-2 * sched
    tu0, tv0 = torch.tensor(u0, requires_grad=True), torch.tensor(v0, requires_grad=True)
    tsch, tpar = torch.tensor(sched, requires_grad=True), torch.tensor(params, requires_grad=True)
    i0 = None
    loss = trajectory_loss(system, tu0, tv0, tsch, tpar, K=K, last=LAST)
    loss.backward()
    g = [x.grad.clone() for x in (tu0, tv0, tsch, tpar)]

    # torch reference, with the same wells (the run must not change wells)
    system.set_parameters(*params)
    system.u = u0
    i0 = system.chunk.index_at_align.copy()
    ru0, rv0 = torch.tensor(u0, requires_grad=True), torch.tensor(v0, requires_grad=True)
    rsch, rpar = torch.tensor(sched, requires_grad=True), torch.tensor(params, requires_grad=True)
    ref = torch_loss(kind, system, ru0, rv0, rsch, rpar)
    ref.backward()
    r = [x.grad for x in (ru0, rv0, rsch, rpar)]
    system.set_parameters(*params)
    system.u = u0
    system.v = v0
    system.a = np.zeros(N)
    system.adjoint_forward(sched, K=K, last=LAST)
    assert np.array_equal(system.chunk.index_at_align, i0), "wells changed during the run"
    assert abs(loss.item() - ref.item()) <= 1e-12 * abs(ref.item())
    for a, b, name in zip(g, r, ["u0", "v0", "schedule", "params"]):
        err = torch.linalg.norm(a - b) / torch.linalg.norm(b)
        assert err < 1e-9, (name, float(err))


@pytest.mark.parametrize("kind", ["Smooth", "SemiSmooth"])
def test_adjoint_finite_differences(kind):
    system = make(kind)
    u0, v0, sched, params = inputs(1)

    def L(u, v, s, p):
        system.set_parameters(*p)
        system.u = u
        system.v = v
        system.a = np.zeros(N)
        return system.adjoint_forward(s, K=K, last=LAST)

    L(u0, v0, sched, params)
    gu, gv, gs, gp = system.adjoint_backward()
    rng = np.random.default_rng(7)
    h = 1e-6
    for name, g, x in [("u0", gu, u0), ("v0", gv, v0), ("schedule", gs, sched)]:
        d = rng.normal(size=x.shape)
        d /= np.linalg.norm(d)
        plus = [u0, v0, sched]
        minus = [u0, v0, sched]
        i = ["u0", "v0", "schedule"].index(name)
        plus = [y + h * d if j == i else y for j, y in enumerate(plus)]
        minus = [y - h * d if j == i else y for j, y in enumerate(minus)]
        fd = (L(*plus, params) - L(*minus, params)) / (2 * h)
        an = float(np.dot(g, d))
        assert abs(fd - an) <= 1e-6 * max(abs(an), np.linalg.norm(g) * 1e-3), (name, fd, an)
    for i, name in enumerate(["mu", "k_interactions", "eta"]):
        e = np.zeros(3)
        e[i] = h
        fd = (L(u0, v0, sched, params + e) - L(u0, v0, sched, params - e)) / (2 * h)
        assert abs(fd - gp[i]) <= 1e-6 * max(abs(gp[i]), 1e-12), (name, fd, gp[i])


def test_adjoint_leaves_final_state():
    system = make("Smooth")
    u0, v0, sched, params = inputs(2)
    system.set_parameters(*params)
    system.u = u0
    system.v = v0
    system.a = np.zeros(N)
    system.adjoint_forward(sched, K=K, last=LAST)
    uT = system.u
    system.adjoint_backward()
    assert np.array_equal(system.u, uT)
    assert system.u_frame == sched[-1]


def test_autograd_cuda_tensors():
    """CUDA tensors on the system's device go through the device entry points (no host round trip of
    u0, v0 or their gradients) and give the same loss and gradients, bit for bit, as host tensors."""
    system = make("Smooth")
    u0, v0, sched, params = inputs(4)
    out = []
    for dev in ("cpu", "cuda:0"):
        tu0 = torch.tensor(u0, device=dev, requires_grad=True)
        tv0 = torch.tensor(v0, device=dev, requires_grad=True)
        tsch = torch.tensor(sched, device=dev, requires_grad=True)
        tpar = torch.tensor(params, device=dev, requires_grad=True)
        loss = trajectory_loss(system, tu0, tv0, tsch, tpar, K=K, last=LAST)
        loss.backward()
        assert tu0.grad.device == tu0.device and tv0.grad.device == tv0.device
        out.append([loss.detach().cpu()] + [x.grad.detach().cpu() for x in (tu0, tv0, tsch, tpar)])
    for a, b in zip(*out):
        assert torch.equal(a, b)
