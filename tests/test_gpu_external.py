"""External generalized forces (Fem3DRepresentation::addExternalGeneralizedForce, applied by
FemRepresentation::computeFMDK and cleared by DeformableRepresentation::afterUpdate) on the GPU against
the oracle."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu

KW = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _loads(s, npe, seed, count=4):
    """Forces at `count` elements, one of them touching the fixed bottom face, with stiffness and
    damping on some."""
    rng = np.random.default_rng(seed)
    E = s.mesh.num_tets
    bc_nodes = set((s.mesh.bc_dofs // 3).tolist())
    touching = [e for e in range(E) if bc_nodes & set(s.mesh.tets[e].tolist())]
    els = list(rng.choice(E, count - 1, replace=False)) + [touching[0]]
    out = []
    for k, e in enumerate(els):
        c = rng.uniform(0.1, 1.0, npe)
        c /= c.sum()
        F = rng.normal(0, 5.0, 3)
        K = rng.normal(0, 50.0, (3, 3)) if k % 2 == 0 else None
        D = rng.normal(0, 0.5, (3, 3)) if k != 1 else None
        out.append((int(e), c, F, K, D))
    return out


def _pair(precision, element_type=0, steps=3, tol=1e-12, **over):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    if element_type == 2:
        s = mesh.scene_hex_cube(3, 3, 4, seed=4, jitter=0.1)
        npe = 8
    else:
        s = mesh.scene_cube(3, 3, 4, seed=4)
        npe = 4
    kw = dict(KW, cg_tolerance=tol, **over)
    b = Body(s.mesh, precision=precision, element_type=element_type, **kw)
    o = O.OracleModel(s.mesh, element_type=element_type, **kw)
    rng = np.random.default_rng(9)
    v = rng.normal(0, 0.02, b.n)
    v[s.mesh.bc_dofs] = 0.0
    b.set_state(None, v)
    o.set_state(None, v)
    return s, b, o, npe


@pytest.mark.parametrize("precision,tol", [(_lib.PRECISION_FP64, 1e-8), (_lib.PRECISION_MIXED, 1e-6)])
@pytest.mark.parametrize("element_type", [0, 1, 2])
def test_external_forces_match_oracle_and_clear(gpu_lib, precision, tol, element_type):
    s, b, o, npe = _pair(precision, element_type, tol=1e-12 if precision == _lib.PRECISION_FP64 else 1e-10)
    x0 = s.mesh.nodes.ravel()
    for step in range(3):
        if step in (0, 2):
            for e, c, F, K, D in _loads(s, npe, seed=step):
                b.add_external_force(e, c, F, K, D)
                o.add_external_force(e, c, F, K, D)
        assert b.step(1e-3) == _lib.GBFEM_OK
        assert o.step(1e-3) == 0
        x, v = b.state()
        ox, ov = o.state()
        assert rel(x - x0, ox - x0) <= tol, (step, rel(x - x0, ox - x0))
        assert np.all(x[s.mesh.bc_dofs] == x0[s.mesh.bc_dofs])


def test_external_forces_with_newton_iterations(gpu_lib):
    s, b, o, npe = _pair(_lib.PRECISION_FP64, 0, newton_max_iterations=3, newton_epsilon=1e-12)
    for e, c, F, K, D in _loads(s, npe, seed=5):
        b.add_external_force(e, c, F, K, D)
        o.add_external_force(e, c, F, K, D)
    assert b.step(1e-3) == _lib.GBFEM_OK and o.step(1e-3) == 0
    x0 = s.mesh.nodes.ravel()
    assert rel(b.state()[0] - x0, o.state()[0] - x0) <= 1e-8


@pytest.mark.parametrize("element_type", [0, 1])
def test_external_forces_then_graph_steps_equal_plain_steps(gpu_lib, element_type):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(3, 3, 4, seed=4)
    kw = dict(KW, cg_tolerance=1e-10, precision=_lib.PRECISION_MIXED, element_type=element_type)
    a = Body(s.mesh, **kw)
    g = Body(s.mesh, **kw)
    g.set_tuning(*a.tuning())
    for e, c, F, K, D in _loads(s, 4, seed=7):
        a.add_external_force(e, c, F, K, D)
        g.add_external_force(e, c, F, K, D)
    assert a.step(1e-3, 6) == _lib.GBFEM_OK
    assert g.step(1e-3, 6, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    assert np.array_equal(a.state()[0], g.state()[0])


def test_external_force_arguments(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(2, 2, 2)
    b = Body(s.mesh)
    with pytest.raises(_lib.GbfemError):
        b.add_external_force(s.mesh.num_tets, [0.25] * 4, [1.0, 0, 0])
    with pytest.raises(_lib.GbfemError):
        b.add_external_force(-1, [0.25] * 4, [1.0, 0, 0])
