"""Mass lumping (FemRepresentation::setMassLumping; FemRepresentation.cpp:499-508 lumps M for the
system matrix and the Newton mass term, :584-586 the Rayleigh mass force) on the GPU against the
oracle: corotational and linear tetrahedra and hexahedra, FP64 and mixed forms, one and two Newton
iterations, the exported system, graph steps, batches and the adjoint."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu

KW = dict(rayleigh_mass=0.05, rayleigh_stiffness=0.002, gravity=(0, 0, -9.81))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _scene(element_type, seed=4):
    if element_type == 2:
        return mesh.scene_hex_cube(3, 3, 4, seed=seed, jitter=0.1)
    return mesh.scene_cube(3, 3, 4, seed=seed)


def _pair(precision, element_type=0, tol=1e-12, lumping=True, **over):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = _scene(element_type)
    kw = dict(KW, cg_tolerance=tol, **over)
    b = Body(s.mesh, precision=precision, element_type=element_type, mass_lumping=lumping, **kw)
    o = O.OracleModel(s.mesh, element_type=element_type, mass_lumping=lumping, **kw)
    rng = np.random.default_rng(9)
    v = rng.normal(0, 0.02, b.n)
    v[s.mesh.bc_dofs] = 0.0
    b.set_state(None, v)
    o.set_state(None, v)
    return s, b, o


@pytest.mark.parametrize("precision,gate", [(_lib.PRECISION_FP64, 1e-8), (_lib.PRECISION_MIXED, 1e-6)])
@pytest.mark.parametrize("element_type", [0, 1, 2])
@pytest.mark.parametrize("newton", [1, 2])
def test_lumped_steps_match_oracle(gpu_lib, precision, gate, element_type, newton):
    """Displacements within the form's gate (FP64 1e-8, mixed 1e-6); velocities within 1e-8 (FP64)
    and 1e-5 (mixed: each step's velocity increment carries the FP32 tangent's ~1e-7 relative error
    directly, where the displacement integrates it)."""
    s, b, o = _pair(precision, element_type, newton_max_iterations=newton, newton_epsilon=1e-12)
    rest = s.mesh.nodes.ravel()
    vgate = gate if precision == _lib.PRECISION_FP64 else 1e-5
    for _ in range(3):
        assert b.step(1e-3, 10) == _lib.GBFEM_OK
        assert o.step(1e-3, 10) == 0
        gx, gv = b.state()
        ox, ov = o.state()
        assert rel(gx - rest, ox - rest) <= gate
        assert rel(gv, ov) <= vgate


def test_lumping_changes_the_step(gpu_lib):
    """The lumped and consistent bodies differ by far more than the parity gate (the test above
    would not pass with the flag ignored)."""
    _, bl, _ = _pair(_lib.PRECISION_FP64, 0, lumping=True)
    s, bc, _ = _pair(_lib.PRECISION_FP64, 0, lumping=False)
    bl.step(1e-3, 10)
    bc.step(1e-3, 10)
    rest = s.mesh.nodes.ravel()
    assert rel(bl.state()[0] - rest, bc.state()[0] - rest) > 1e-4


def test_lumped_system_export_matches_oracle(gpu_lib):
    """S, rhs and f of a lumped step (GBFEM_STEP_KEEP_SYSTEM) against the oracle's."""
    s, b, o = _pair(_lib.PRECISION_FP64, 0)
    rng = np.random.default_rng(2)
    x = s.mesh.nodes.ravel() + rng.normal(0, 2e-4, b.n)
    x[s.mesh.bc_dofs] = s.mesh.nodes.ravel()[s.mesh.bc_dofs]
    b.set_state(x, None)
    o.set_state(x, None)
    assert b.step(1e-3, 1, _lib.STEP_KEEP_SYSTEM) == _lib.GBFEM_OK
    assert o.step(1e-3, 1) == 0
    gs, os_ = b.system(), o.system()
    assert np.max(np.abs(gs["S"] - os_["S"])) <= 1e-12 * np.max(np.abs(os_["S"]))
    assert rel(gs["rhs"], os_["rhs"]) <= 1e-12
    assert rel(gs["f"], os_["f"]) <= 1e-12


def test_lumped_graph_steps_and_batch(gpu_lib):
    """Mixed graph steps of a lumped batch of two meshes against the oracle (1e-6)."""
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    scenes = [mesh.scene_cube(3, 3, 4, seed=4), mesh.scene_cube(2, 4, 3, seed=5, young=3e5)]
    kw = dict(KW, cg_tolerance=1e-11)
    b = Body([sc.mesh for sc in scenes], precision=_lib.PRECISION_MIXED, mass_lumping=True, **kw)
    assert b.step(1e-3, 12, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    gx, _ = b.state()
    for k, sc in enumerate(scenes):
        o = O.OracleModel(sc.mesh, mass_lumping=True, **kw)
        assert o.step(1e-3, 12) == 0
        n0, n1 = b.node_offsets[k], b.node_offsets[k + 1]
        rest = sc.mesh.nodes.ravel()
        assert rel(gx[3 * n0:3 * n1] - rest, o.state()[0] - rest) <= 1e-6


def _lumped_v0_gradient(torch, precision):
    """(gradient of wx . x_T in v0, the forward as a function of a v0 offset, the data) of a lumped
    5-step rollout."""
    from opensurgsim_gb300.autograd import rollout
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(3, 3, 4, seed=6)
    prec = _lib.PRECISION_MIXED if precision == "mixed" else _lib.PRECISION_FP64
    body = Body(s.mesh, precision=prec, mass_lumping=True, cg_tolerance=1e-13 if precision == "fp64" else 1e-12,
                **KW)
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(12)
    theta = torch.tensor(np.log(s.mesh.young), dtype=torch.float64, device=dev)
    x0 = torch.tensor(s.mesh.nodes.ravel(), dtype=torch.float64, device=dev)
    v0 = torch.tensor(rng.normal(0, 0.01, body.n), dtype=torch.float64, device=dev)
    bc = torch.tensor(s.mesh.bc_dofs, dtype=torch.long, device=dev)
    v0[bc] = 0.0
    wx = torch.tensor(rng.normal(0, 1, body.n), dtype=torch.float64, device=dev)
    v0g = v0.clone().requires_grad_(True)
    xT, _ = rollout(body, theta, x0, v0g, 1e-3, 5, checkpoint_every=2)
    (wx * xT).sum().backward()

    def val(offset):
        with torch.no_grad():
            xT_, _ = rollout(body, theta, x0, v0 + offset, 1e-3, 5, checkpoint_every=2)
            return float((wx * xT_).sum())

    return v0g.grad.detach().clone(), val, bc, body.n


def test_lumped_adjoint_velocity_gradient(gpu_lib):
    """With lumping the adjoint's d psi / d v uses the lumped mass. FP64: the rollout's gradient in v0
    against a central difference of the forward rollout along a random direction (1e-5). Mixed: the
    same gradient against the FP64 adjoint's (1e-4)."""
    torch = pytest.importorskip("torch")
    g64, val, bc, n = _lumped_v0_gradient(torch, "fp64")
    rng = np.random.default_rng(13)
    d = torch.tensor(rng.normal(0, 1, n), dtype=torch.float64, device="cuda:0")
    d[bc] = 0.0
    h = 1e-6
    fd = (val(h * d) - val(-h * d)) / (2 * h)
    ad = float((g64 * d).sum())
    assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)
    g32, _, _, _ = _lumped_v0_gradient(torch, "mixed")
    err = float(torch.linalg.norm(g32 - g64) / torch.linalg.norm(g64))
    assert err <= 1e-4, err
