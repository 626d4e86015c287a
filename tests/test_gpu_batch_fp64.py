"""FP64 batches: many meshes in one handle in the plain FP64 form, every mesh's Eigen CG run in one
persistent FP64 launch (k_pcg_persistent<true>), against the oracle and against one FP64 handle per
mesh (whose CG runs with separate launches per iteration)."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu

KW = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0.0, 0.0, -9.81), cg_tolerance=1e-10)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _scenes():
    return [mesh.scene_cube(3, 3, 4, seed=1, young=3e4), mesh.scene_cube(6, 5, 7, seed=2, young=4e5),
            mesh.scene_cube(2, 2, 2, seed=3, young=1e5), mesh.scene_cube(5, 4, 3, seed=4, young=8e5)]


def _split(body, x, k):
    n0, n1 = body.node_offsets[k], body.node_offsets[k + 1]
    return x[3 * n0:3 * n1]


@pytest.mark.parametrize("graph", [False, True])
def test_fp64_batch_matches_oracle_and_single_handles(gpu_lib, graph):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    scenes = _scenes()
    batch = Body([s.mesh for s in scenes], precision=_lib.PRECISION_FP64, **KW)
    flags = _lib.STEP_GRAPH if graph else 0
    assert batch.step(1e-3, 20, flags) == _lib.GBFEM_OK
    seg = batch.segment_stats()
    bx, bv = batch.state()
    for k, s in enumerate(scenes):
        rest = s.mesh.nodes.ravel()
        o = O.OracleModel(s.mesh, **KW)
        assert o.step(1e-3, 20) == 0
        ox, ov = o.state()
        assert rel(_split(batch, bx, k) - rest, ox - rest) <= 1e-8
        # Velocities at 1e-6: the small stiff mesh is near rest under gravity after 20 steps (|v| ~ 1e-9
        # m/s), where the CG's tolerance relative to the step's right-hand side sets their digits.
        assert rel(_split(batch, bv, k), ov) <= 1e-6
        single = Body(s.mesh, precision=_lib.PRECISION_FP64, **KW)
        its = 0
        for _ in range(20):
            assert single.step(1e-3, 1) == _lib.GBFEM_OK
            its += single.stats()["cg_iterations"]
        sx, _ = single.state()
        assert rel(_split(batch, bx, k) - rest, sx - rest) <= 1e-9
        # Same Eigen iteration and stopping rule; sums in another order may move a stop by one.
        assert abs(int(seg["iterations"][k]) - its) <= 20, (k, seg["iterations"][k], its)
        assert seg["converged"][k] == 1
        assert seg["refreshes"][k] == 0


def test_fp64_batch_graph_steps_equal_plain_steps(gpu_lib):
    from opensurgsim_gb300.body import Body

    scenes = _scenes()
    out = []
    for flags in (0, _lib.STEP_GRAPH):
        b = Body([s.mesh for s in scenes], precision=_lib.PRECISION_FP64, **KW)
        b.set_tuning(64, 3, 2)  # pinned: the partition sets the rounding of the solve's sums
        assert b.step(1e-3, 12, flags) == _lib.GBFEM_OK
        out.append(b.state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_fp64_batch_autotunes_and_adjoint_runs(gpu_lib):
    """The autotuner picks the FP64 solve's CTAs per SM among those that fit; the adjoint
    step of a batch solves its transposed system with the same persistent launch and matches the
    mixed batch's gradient within 1e-4."""
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300.autograd import rollout
    from opensurgsim_gb300.body import Body

    scenes = _scenes()
    b = Body([s.mesh for s in scenes], precision=_lib.PRECISION_FP64, autotune=True, **KW)
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    eb, cps, rw, sched = b.tuning()
    assert cps in (1, 2, 3, 4) and sched == _lib.CG_FP64
    grads = {}
    dev = torch.device("cuda:0")
    for prec in ("fp64", "mixed"):
        kw = dict(KW, cg_tolerance=1e-12)
        body = Body([s.mesh for s in scenes], precision=_lib.PRECISION_FP64 if prec == "fp64" else
                    _lib.PRECISION_MIXED, **kw)
        young = np.concatenate([s.mesh.young for s in scenes])
        theta = torch.tensor(np.log(young), dtype=torch.float64, device=dev).requires_grad_(True)
        x0 = torch.tensor(np.concatenate([s.mesh.nodes.ravel() for s in scenes]), dtype=torch.float64, device=dev)
        rng = np.random.default_rng(3)
        v0 = torch.zeros(body.n, dtype=torch.float64, device=dev)
        w = torch.tensor(rng.normal(0, 1, body.n), dtype=torch.float64, device=dev)
        xT, _ = rollout(body, theta, x0, v0, 1e-3, 6, checkpoint_every=3)
        (w * (xT - x0)).sum().backward()
        grads[prec] = theta.grad.detach().cpu().numpy()
    err = np.linalg.norm(grads["mixed"] - grads["fp64"]) / np.linalg.norm(grads["fp64"])
    assert err <= 1e-4, err
