"""Adjoint of the FP64 step (ch_adjoint) with frozen collision events.

Checked three ways on a small plasma (the differentiation workload's
physics: E0 = (0.5, 0.1, 0), nu = 0.3, 0.01 sin(2 pi x / Lx) loading):
  * against central finite differences of the GPU forward replay
    (the same frozen events): agreement to 1e-5 relative;
  * against the FP64 oracle's replay of the exported events (an independent
    CPU implementation of the frozen-event model): J to 1e-9, and its
    central-difference gradient against the adjoint to 1e-5;
  * through the torch.autograd.Function binding.
Relative errors are per component against max(|g_k|, 1e-3 ||g||).

The GPU replay's differences use one stated step for every component,
eps = 1e-7 (the oracle replay's, below, 1e-6).
The amplitude perturbation moves every ion's initial position by
eps dx0/damp, at most 2 Lx / (2 pi) / 0.99 eps (5e-7 cells on the 16^3 grid),
and an ion that comes that close to a cell face in any step passes a kink of
the CIC weights, which biases its difference quotient.  The expected number
of such ion-steps is 2 x 5e-7 per ion-step x 32768 ions x 12 steps = 0.4, so
the differences see smooth functions.  The noise of J (solves to rtol
1e-13) is about 1e-15, or 5e-9 in a difference quotient.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS = 1e-7
RTOL_SOLVE = 1e-13


def _central(f, th, g, eps=EPS):
    """Central differences of f at th, the same step for every component."""
    fd = np.empty_like(g)
    for k in range(len(th)):
        e = np.zeros_like(th)
        e[k] = eps
        fd[k] = (f(th + e) - f(th - e)) / (2 * eps)
    return fd


def _setup(chy, N=(16, 16, 16), ppc=8, nsteps=12, every=4, window=4, seed=5):
    p = chy.params_for(N, precision=chy.PRECISION["fp64"], E0=(0.5, 0.1, 0.0), nui=0.3, ksp_rtol=RTOL_SOLVE,
                       pc_type=chy.PC["mg"], seed=seed)
    L = chy.loader(amp=(0.01, 0.0, 0.0))
    np_ = N[0] * N[1] * N[2] * ppc
    return p, L, np_, dict(nsteps=nsteps, checkpoint_every=every, window=window)


def _rel_err(g, ref):
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    return np.abs(g - ref) / scale


def test_adjoint_matches_central_differences(chy):
    p, L, np_, cfg = _setup(chy)
    with chy.Adjoint(p, np_, L, **cfg) as adj:
        th = adj.theta0()
        J0 = adj.forward(th, record=True)
        g, Jg = adj.gradient()
        assert Jg == J0
        # replay at the recorded point reproduces J exactly
        assert adj.forward(th) == J0
        fd = _central(adj.forward, th, g)
        err = _rel_err(g, fd)
        assert err.max() < 1e-5, (g, fd, err)
        # every parameter matters in this plasma
        assert np.all(np.abs(fd) > 1e-8 * np.abs(fd).max())
        t = adj.timing()
        assert t["events"] > 0 and t["gradient_ms"] > 0


def test_adjoint_checkpoint_interval_does_not_change_the_gradient(chy):
    p, L, np_, cfg = _setup(chy, nsteps=9, every=3, window=3)
    out = []
    for every in (1, 3, 9):
        cfg["checkpoint_every"] = every
        with chy.Adjoint(p, np_, L, **cfg) as adj:
            adj.forward(adj.theta0(), record=True)
            out.append(adj.gradient()[0])
    assert np.abs(out[1] - out[0]).max() <= 1e-12 * np.abs(out[0]).max()
    assert np.abs(out[2] - out[0]).max() <= 1e-12 * np.abs(out[0]).max()


def test_adjoint_against_fp64_oracle_replay(chy, po):
    p, L, np_, cfg = _setup(chy, N=(12, 12, 12), ppc=6, nsteps=8, every=4, window=3, seed=9)
    q = po.params_from(p)
    with chy.Adjoint(p, np_, L, **cfg) as adj:
        th = adj.theta0()
        J = adj.forward(th, record=True)
        g, _ = adj.gradient()
        ev = adj.events()
    assert len(ev["step"]) > 0

    def oracle_J(theta):
        q.E0[:] = theta[0:3]
        q.vn0[:] = theta[3:6]
        Lo = po.make_loader(amp=(theta[6], 0.0, 0.0))
        return po.adj_objective(q, Lo, np_, cfg["nsteps"], cfg["window"], 1.0, 0.1, ev, RTOL_SOLVE)

    Jo = oracle_J(th)
    assert abs(Jo - J) <= 1e-9 * abs(J), (Jo, J)
    # the oracle's Jacobi-CG solves leave about 4e-14 of noise in J, so its
    # differences take eps = 1e-6 for every component; on this 12^3 case
    # that moves ions by at most 4e-6 cells: 2 x 4e-6 x 10368 ions x 8
    # steps = 0.7 expected kink ion-steps
    fd = _central(oracle_J, th, g, eps=1e-6)
    err = _rel_err(g, fd)
    assert err.max() < 1e-5, (g, fd, err)


def test_torch_autograd_binding(chy):
    torch = pytest.importorskip("torch")
    import importlib

    ag = importlib.import_module("collisional-hybrid_gb300.autograd")
    p, L, np_, cfg = _setup(chy, nsteps=6, every=3, window=2)
    with chy.Adjoint(p, np_, L, **cfg) as adj:
        theta = torch.tensor(adj.theta0(), dtype=torch.float64, requires_grad=True)
        J = ag.objective(theta, adj)
        J.backward()
        # a second reverse sweep of the same recorded run gives the same gradient
        g, Jg = adj.gradient()
        assert float(J.detach()) == Jg
        assert np.allclose(theta.grad.numpy(), g, rtol=1e-12, atol=0.0)
