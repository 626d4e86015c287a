"""Differentiation form on the GPU: gradients of a multi-step rollout (gbfem_adjoint_step behind
torch.autograd) against central finite differences of the forward rollout, FP64 and mixed."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _setup(precision, nx=3, ny=3, nz=4, tol=1e-13, seed=0):
    from opensurgsim_gb300 import _lib, mesh
    from opensurgsim_gb300.body import Body

    scene = mesh.scene_cube(nx, ny, nz, seed=seed)
    prec = _lib.PRECISION_MIXED if precision == "mixed" else _lib.PRECISION_FP64
    body = Body.from_scene(scene, precision=prec, cg_tolerance=tol)
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(seed + 11)
    m = scene.mesh
    theta = torch.tensor(np.log(m.young) + rng.normal(0, 0.3, m.num_tets), dtype=torch.float64, device=dev)
    x0 = torch.tensor(m.nodes.ravel(), dtype=torch.float64, device=dev)
    v0 = torch.tensor(rng.normal(0, 0.01, body.n), dtype=torch.float64, device=dev)
    v0[torch.tensor(m.bc_dofs, dtype=torch.long, device=dev)] = 0.0
    wx = torch.tensor(rng.normal(0, 1, body.n), dtype=torch.float64, device=dev)
    wv = torch.tensor(rng.normal(0, 1e-3, body.n), dtype=torch.float64, device=dev)
    return scene, body, theta, x0, v0, wx, wv


def _loss(body, theta, x0, v0, wx, wv, dt, steps, every=4, nu=None):
    from opensurgsim_gb300.autograd import rollout

    xT, vT = rollout(body, theta, x0, v0, dt, steps, checkpoint_every=every, poisson=nu)
    return (wx * (xT - x0)).sum() + (wv * vT).sum()


def _loss_value(body, theta, x0, v0, wx, wv, dt, steps, nu=None):
    with torch.no_grad():
        return float(_loss(body, theta, x0, v0, wx, wv, dt, steps, nu=nu))


def _poisson(scene, seed):
    """Per-element Poisson ratios around the scene's 0.45 (float64 on cuda:0)."""
    rng = np.random.default_rng(seed + 23)
    nu = scene.mesh.poisson + rng.uniform(-0.03, 0.03, scene.mesh.num_tets)
    return torch.tensor(nu, dtype=torch.float64, device="cuda:0")


@pytest.mark.parametrize("steps,every", [(6, 4), (5, 10)])
def test_fp64_log_young_gradient_matches_central_differences(gpu_lib, steps, every):
    scene, body, theta, x0, v0, wx, wv = _setup("fp64")
    th = theta.clone().requires_grad_(True)
    L = _loss(body, th, x0, v0, wx, wv, scene.dt, steps, every)
    L.backward()
    g = th.grad.detach().cpu().numpy()
    h = 1e-5
    fd = np.zeros_like(g)
    for e in range(g.size):
        tp, tm = theta.clone(), theta.clone()
        tp[e] += h
        tm[e] -= h
        fd[e] = (_loss_value(body, tp, x0, v0, wx, wv, scene.dt, steps) -
                 _loss_value(body, tm, x0, v0, wx, wv, scene.dt, steps)) / (2 * h)
    err = np.linalg.norm(g - fd) / np.linalg.norm(fd)
    assert err <= 1e-4, err
    big = np.abs(fd) > 0.1 * np.abs(fd).max()
    assert np.max(np.abs(g[big] - fd[big]) / np.abs(fd[big])) <= 1e-3


def test_fp64_initial_state_gradients_match_directional_differences(gpu_lib):
    scene, body, theta, x0, v0, wx, wv = _setup("fp64", seed=4)
    from opensurgsim_gb300.autograd import rollout

    x0g = x0.clone().requires_grad_(True)
    v0g = v0.clone().requires_grad_(True)
    xT, vT = rollout(body, theta, x0g, v0g, scene.dt, 5, checkpoint_every=2)
    L = (wx * xT).sum() + (wv * vT).sum()
    L.backward()
    rng = np.random.default_rng(7)
    bc = torch.tensor(scene.mesh.bc_dofs, dtype=torch.long, device=x0.device)
    for which, base, grad in (("v", v0, v0g.grad), ("x", x0, x0g.grad)):
        d = torch.tensor(rng.normal(0, 1, body.n), dtype=torch.float64, device=x0.device)
        d[bc] = 0.0
        h = 1e-6 if which == "v" else 1e-8

        def val(delta):
            with torch.no_grad():
                xa = x0 + delta * d if which == "x" else x0
                va = v0 + delta * d if which == "v" else v0
                xT_, vT_ = rollout(body, theta, xa, va, scene.dt, 5, checkpoint_every=2)
                return float((wx * xT_).sum() + (wv * vT_).sum())

        fd = (val(h) - val(-h)) / (2 * h)
        ad = float((grad * d).sum())
        assert abs(ad - fd) <= 1e-5 * abs(fd), (which, ad, fd)


def test_mixed_adjoint_agrees_with_fp64_adjoint(gpu_lib):
    grads = {}
    for prec in ("fp64", "mixed"):
        scene, body, theta, x0, v0, wx, wv = _setup(prec, tol=1e-12, seed=2)
        th = theta.clone().requires_grad_(True)
        _loss(body, th, x0, v0, wx, wv, scene.dt, 6).backward()
        grads[prec] = th.grad.detach().cpu().numpy()
    err = np.linalg.norm(grads["mixed"] - grads["fp64"]) / np.linalg.norm(grads["fp64"])
    assert err <= 1e-4, err


def test_adjoint_is_deterministic(gpu_lib):
    out = []
    for _ in range(2):
        scene, body, theta, x0, v0, wx, wv = _setup("fp64", seed=5)
        th = theta.clone().requires_grad_(True)
        _loss(body, th, x0, v0, wx, wv, scene.dt, 4).backward()
        out.append(th.grad.detach().cpu().numpy())
    assert np.array_equal(out[0], out[1])


def test_fp64_poisson_gradient_matches_central_differences(gpu_lib):
    """dL/d nu_e of the rollout (grad_poisson of gbfem_adjoint_step through autograd) against
    central differences of the forward rollout in nu_e, on 40 random elements, with log E
    differentiated in the same backward pass."""
    scene, body, theta, x0, v0, wx, wv = _setup("fp64", seed=6)
    nu = _poisson(scene, 6)
    th = theta.clone().requires_grad_(True)
    nug = nu.clone().requires_grad_(True)
    L = _loss(body, th, x0, v0, wx, wv, scene.dt, 6, nu=nug)
    L.backward()
    g = nug.grad.detach().cpu().numpy()
    assert th.grad is not None and torch.isfinite(th.grad).all()
    rng = np.random.default_rng(3)
    sel = rng.choice(g.size, 40, replace=False)
    h = 1e-5
    fd = np.zeros(sel.size)
    for i, e in enumerate(sel):
        npl, nmi = nu.clone(), nu.clone()
        npl[e] += h
        nmi[e] -= h
        fd[i] = (_loss_value(body, theta, x0, v0, wx, wv, scene.dt, 6, nu=npl) -
                 _loss_value(body, theta, x0, v0, wx, wv, scene.dt, 6, nu=nmi)) / (2 * h)
    err = np.linalg.norm(g[sel] - fd) / np.linalg.norm(fd)
    assert err <= 1e-4, err


def test_mixed_poisson_gradient_agrees_with_fp64_adjoint(gpu_lib):
    grads = {}
    for prec in ("fp64", "mixed"):
        scene, body, theta, x0, v0, wx, wv = _setup(prec, tol=1e-12, seed=8)
        nug = _poisson(scene, 8).requires_grad_(True)
        _loss(body, theta, x0, v0, wx, wv, scene.dt, 6, nu=nug).backward()
        grads[prec] = nug.grad.detach().cpu().numpy()
    err = np.linalg.norm(grads["mixed"] - grads["fp64"]) / np.linalg.norm(grads["fp64"])
    assert err <= 1e-4, err


def _graph_case(seed=9):
    scene, body, theta, x0, v0, wx, wv = _setup("mixed", tol=1e-12, seed=seed)
    nu = _poisson(scene, seed)
    return scene, body, theta, nu, x0, v0, wx, wv


def _grads(body, theta, nu, x0, v0, wx, wv, dt, steps=7, every=3):
    th = theta.clone().requires_grad_(True)
    nug = nu.clone().requires_grad_(True)
    x0g = x0.clone().requires_grad_(True)
    v0g = v0.clone().requires_grad_(True)
    from opensurgsim_gb300.autograd import rollout

    xT, vT = rollout(body, th, x0g, v0g, dt, steps, checkpoint_every=every, poisson=nug)
    ((wx * (xT - x0)).sum() + (wv * vT).sum()).backward()
    return [t.detach().cpu().numpy() for t in (xT, vT, th.grad, nug.grad, x0g.grad, v0g.grad)]


def test_graph_rollout_equals_the_per_step_rollout(gpu_lib, monkeypatch):
    """The mixed form's rollouts run as two CUDA graphs in the library (gbfem_rollout_forward /
    _backward); the same rollout through the per-step loop (gbfem_step and gbfem_adjoint_step from
    Python) gives the same states and gradients bit for bit (the same kernels in the same order)."""
    from opensurgsim_gb300 import autograd

    scene, body, theta, nu, x0, v0, wx, wv = _graph_case()
    assert autograd.graph_rollouts(body)
    body.set_tuning(64, 4, 2)  # one partition for both runs
    g = _grads(body, theta, nu, x0, v0, wx, wv, scene.dt)
    monkeypatch.setattr(autograd, "graph_rollouts", lambda b: False)
    ref = _grads(body, theta, nu, x0, v0, wx, wv, scene.dt)
    for a, b in zip(g, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("graph", [True, False])
def test_rollout_keeping_every_state_equals_segment_reruns(gpu_lib, monkeypatch, graph):
    """checkpoint_every=1 keeps every state, so the reverse sweep re-runs no step; its states and
    gradients equal those of checkpoints every 3 steps (whose segments re-run their steps, with the
    same deterministic kernels) bit for bit, in the library's graph rollouts and in the per-step loop."""
    from opensurgsim_gb300 import autograd

    scene, body, theta, nu, x0, v0, wx, wv = _graph_case(seed=12)
    body.set_tuning(64, 4, 2)
    if not graph:
        monkeypatch.setattr(autograd, "graph_rollouts", lambda b: False)
    g1 = _grads(body, theta, nu, x0, v0, wx, wv, scene.dt, steps=7, every=1)
    g3 = _grads(body, theta, nu, x0, v0, wx, wv, scene.dt, steps=7, every=3)
    for a, b in zip(g1, g3):
        assert np.array_equal(a, b)


def test_graph_rollout_backward_after_another_forward(gpu_lib):
    """The library keeps the checkpoints of the body's last forward; a backward whose forward was
    followed by another rollout of the same body runs its forward again and gives the gradient of a
    backward taken right away."""
    from opensurgsim_gb300.autograd import rollout

    scene, body, theta, nu, x0, v0, wx, wv = _graph_case(seed=10)
    th = theta.clone().requires_grad_(True)
    xT, _ = rollout(body, th, x0, v0, scene.dt, 6, checkpoint_every=4)
    (wx * xT).sum().backward()
    want = th.grad.detach().clone()
    th2 = theta.clone().requires_grad_(True)
    xA, _ = rollout(body, th2, x0, v0, scene.dt, 6, checkpoint_every=4)
    with torch.no_grad():
        rollout(body, theta + 0.1, x0, v0 * 2, scene.dt, 6, checkpoint_every=4)  # another forward in between
    (wx * xA).sum().backward()
    assert torch.equal(th2.grad, want)
