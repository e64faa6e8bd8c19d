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


def torch_loss_schedule(kind, data, u0, v0, sched, params, kf, last, kappa=1.0, segment=100):
    """The unrolled FP64 forward in torch on u0's device for any size, in checkpointed segments of
    `segment` steps (autograd recomputes each segment in the backward).  The well of every particle is
    looked up at every step from its chunk row data [N, W] (y[i] <= u < y[i+1], the align rule), so
    particles may change well as in the library's forward; the index has zero derivative."""
    from torch.utils.checkpoint import checkpoint

    mu, k, eta = params[0], params[1], params[2]
    m, dt = 1.0, 0.1
    T = sched.shape[0]

    def seg(u, v, a, acc, t0, t1):
        for t in range(t0, t1):
            up = (u + dt * v) + ((0.5 * dt) * dt) * a
            i = torch.searchsorted(data, up.detach().unsqueeze(1), right=True) - 1
            yl = torch.gather(data, 1, i).squeeze(1)
            yr = torch.gather(data, 1, i + 1).squeeze(1)
            if kind == "Smooth":
                umin = 0.5 * (yl + yr)
                dy = 0.5 * (yr - yl)
                fp = -mu * dy / math.pi * torch.sin(math.pi * (up - umin) / dy)
            else:
                xi = 0.5 * (yl + yr)
                u_r = (mu * xi + kappa * yr) / (mu + kappa)
                u_l = (mu * xi + kappa * yl) / (mu + kappa)
                fp = torch.where(up < u_l, kappa * (up - yl),
                                 torch.where(up <= u_r, mu * (0.5 * (yl + yr) - up), kappa * (up - yr)))
            fi = k * ((torch.roll(up, 1) - 2 * up) + torch.roll(up, -1))
            ff = kf * (sched[t] - up)
            s = (ff + fp) + fi
            v1 = v + dt * a
            a1 = (s + (-eta) * v1) / m
            v2 = v + (0.5 * dt) * (a + a1)
            a2 = (s + (-eta) * v2) / m
            v3 = v + (0.5 * dt) * (a + a2)
            a3 = (s + (-eta) * v3) / m
            if t >= T - last:
                acc = acc + torch.mean(ff)
            u, v, a = up, v3, a3
        return u, v, a, acc

    u, v, a = u0, v0, torch.zeros_like(u0)
    acc = torch.zeros((), dtype=torch.float64, device=u0.device)
    for t0 in range(0, T, segment):
        u, v, a, acc = checkpoint(seg, u, v, a, acc, t0, min(T, t0 + segment), use_reentrant=False)
    return acc / last + 0.5 * torch.mean(u * u)


@pytest.mark.timeout(1800)
@pytest.mark.parametrize("kind", ["Smooth", "SemiSmooth"])
def test_adjoint_full_size(kind):
    """The differentiation workload at its own size: Line1d System_{Smooth,SemiSmooth}_Laplace (kappa = 1),
    N = 65536, m = 1, eta = 0.1, mu = 1, k = 1, k_frame = 1/N, dt = 0.1, Weibull(2,1)+1e-5 from pcg32
    seed 4, T = 5000 steps with u_frame(t) = 1e-3 t + 0.05 sin(2 pi t / 500), loss = mean f_frame over
    the last 500 steps + 0.5 mean(u_T^2), checkpoints every 100 steps; u0 = the equilibrium at
    u_frame = 0 (minimise from u = v = 0), v0 = 0.  (From u = 0 itself many particles start near a
    potential maximum and fall to either side: the loss then changes by finite amounts under 1e-6
    perturbations, and no finite difference resolves a derivative.)  A few particles still change well
    during the run (quasistatic slips).
    (1) Against torch autograd through the unrolled FP64 step on the GPU, with every particle's well
    looked up at every step as the forward does: relative error of every gradient below 1e-9.
    (2) Against central finite differences of the library's forward, h = 1e-6: along mu,
    k_interactions and eta, and along one random direction (entries uniform in [0, 1)) of u0, v0 and
    the schedule, within 1e-6 relative plus the finite difference's own resolution, 64 ulp(loss) / h
    (the loss sums 500 x 65536 frame forces, so its rounding reaches a few dozen ulp)."""
    N, T, Kc, last = 65536, 5000, 100, 500
    par = dict(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / N, dt=0.1, shape=[N], seed=4,
               distribution="weibull", parameters=[2.0, 1.0, 1e-5], offset=-100.0, nchunk=1000)
    system = (fqsb.Line1d.System_Smooth_Laplace(**par) if kind == "Smooth"
              else fqsb.Line1d.System_SemiSmooth_Laplace(kappa=1.0, **par))
    system.minimise(max_iter=1000000)
    ueq = system.u
    t = np.arange(T)
    sched = 1e-3 * t + 0.05 * np.sin(2 * np.pi * t / 500)
    params = np.array([1.0, 1.0, 0.1])
    zero = np.zeros(N)

    def L(u0=ueq, v0=zero, sc=sched, p=params):
        system.set_parameters(*p)
        system.u, system.v, system.a = u0, v0, zero
        return system.adjoint_forward(sc, K=Kc, last=last)

    system.u = ueq
    start = system.chunk.start.copy()
    data = torch.tensor(system.chunk.data, dtype=torch.float64, device="cuda")
    L0 = L()
    assert np.array_equal(system.chunk.start, start), "a chunk window moved: the torch restatement reads one window"
    gu, gv, gs, gp = system.adjoint_backward()

    tu0 = torch.tensor(ueq, device="cuda", requires_grad=True)
    tv0 = torch.zeros(N, dtype=torch.float64, device="cuda", requires_grad=True)
    tsch = torch.tensor(sched, device="cuda", requires_grad=True)
    tpar = torch.tensor(params, device="cuda", requires_grad=True)
    ref = torch_loss_schedule(kind, data, tu0, tv0, tsch, tpar, 1.0 / N, last)
    ref.backward()
    assert abs(L0 - ref.item()) <= 1e-12 * abs(ref.item())
    for a, b, name in zip([gu, gv, gs, gp], [tu0.grad, tv0.grad, tsch.grad, tpar.grad],
                          ["u0", "v0", "schedule", "params"]):
        b = b.cpu().numpy()
        err = np.linalg.norm(a.ravel() - b.ravel()) / np.linalg.norm(b)
        assert err < 1e-9, (name, err)

    h = 1e-6
    noise = 64 * np.spacing(abs(L0)) / h
    for i, name in enumerate(["mu", "k_interactions", "eta"]):
        e = np.zeros(3)
        e[i] = h
        fd = (L(p=params + e) - L(p=params - e)) / (2 * h)
        assert abs(fd - gp[i]) <= 1e-6 * abs(gp[i]) + noise, (name, fd, gp[i], noise)
    rng = np.random.default_rng(9)
    for name, g, x in [("u0", gu, ueq), ("v0", gv, zero), ("sc", gs, sched)]:
        d = rng.uniform(0.0, 1.0, x.shape)
        fd = (L(**{name: x + h * d}) - L(**{name: x - h * d})) / (2 * h)
        an = float(np.dot(g.ravel(), d.ravel()))
        assert abs(fd - an) <= 1e-6 * abs(an) + noise, (name, fd, an, noise)
