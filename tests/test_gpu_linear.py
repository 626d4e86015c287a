"""Linear tetrahedron path (Fem3DElementTetrahedron + OdeSolverLinearEulerImplicit) on the GPU
against the oracle's linear element."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _pair(precision, steps=40, seed=2, tol=1e-12):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(4, 4, 6, seed=seed, young=2e5)
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=tol)
    b = Body(s.mesh, precision=precision, element_type=_lib.ELEMENT_LINEAR_TET, **kw)
    o = O.OracleModel(s.mesh, element_type=1, **kw)
    v0 = np.random.default_rng(seed).normal(0, 0.02, b.n)
    v0[s.mesh.bc_dofs] = 0.0
    b.set_state(None, v0)
    o.set_state(None, v0)
    launches = []
    for _ in range(steps):
        assert b.step(1e-3) == _lib.GBFEM_OK
        launches.append(b.stats()["kernel_launches"])
        assert o.step(1e-3) == 0
    return s, b, o, launches


def test_linear_fp64_matches_oracle_and_reuses_the_system(gpu_lib):
    s, b, o, launches = _pair(_lib.PRECISION_FP64)
    x, v = b.state()
    ox, ov = o.state()
    x0 = s.mesh.nodes.ravel()
    assert rel(x - x0, ox - x0) <= 1e-8
    assert rel(v, ov) <= 1e-8


def test_linear_mixed_matches_oracle_and_reuses_the_system(gpu_lib):
    s, b, o, launches = _pair(_lib.PRECISION_MIXED, tol=1e-10)
    x, _ = b.state()
    ox, _ = o.state()
    x0 = s.mesh.nodes.ravel()
    assert rel(x - x0, ox - x0) <= 1e-6
    # The first step assembles; the later ones update the right-hand side only (one launch fewer).
    assert launches[0] == launches[1] + 1 and all(l == launches[1] for l in launches[2:])


def test_linear_reuse_equals_fresh_assembly(gpu_lib):
    """A step with the stored linear system equals a step of a handle that assembles afresh."""
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(3, 3, 4, seed=5)
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=1e-12,
              element_type=_lib.ELEMENT_LINEAR_TET)
    a = Body(s.mesh, **kw)
    for _ in range(5):
        assert a.step(1e-3) == _lib.GBFEM_OK
    x, v = a.state()
    fresh = Body(s.mesh, **kw)
    fresh.set_state(x, v)
    assert a.step(1e-3) == _lib.GBFEM_OK
    assert fresh.step(1e-3) == _lib.GBFEM_OK
    assert np.array_equal(a.state()[0], fresh.state()[0])


def test_linear_material_change_rebuilds_the_system(gpu_lib):
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(3, 3, 4, seed=6, young=1e5)
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=1e-12,
              element_type=_lib.ELEMENT_LINEAR_TET)
    a = Body(s.mesh, **kw)
    assert a.step(1e-3, 3) == _lib.GBFEM_OK
    x, v = a.state()
    E2 = torch.full((s.mesh.num_tets,), 3e5, dtype=torch.float64, device="cuda:0")
    import ctypes
    torch.cuda.synchronize()
    assert _lib.load().gbfem_set_materials_device(a.handle, ctypes.c_void_p(E2.data_ptr()), None) == 0
    s2 = mesh.scene_cube(3, 3, 4, seed=6, young=3e5)
    b = Body(s2.mesh, **kw)
    b.set_state(x, v)
    assert a.step(1e-3, 2) == _lib.GBFEM_OK
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    x0 = s.mesh.nodes.ravel()
    assert rel(a.state()[0] - x0, b.state()[0] - x0) <= 1e-12


def test_linear_graph_steps_equal_regular_steps(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(4, 3, 5, seed=7)
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=1e-10,
              precision=_lib.PRECISION_MIXED, element_type=_lib.ELEMENT_LINEAR_TET)
    a = Body(s.mesh, **kw)
    g = Body(s.mesh, **kw)
    g.set_tuning(*a.tuning())
    assert a.step(1e-3, 6) == _lib.GBFEM_OK
    assert g.step(1e-3, 6, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    assert np.array_equal(a.state()[0], g.state()[0])


def test_adjoint_rejects_linear_elements(gpu_lib):
    import ctypes

    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(2, 2, 2)
    b = Body(s.mesh, element_type=_lib.ELEMENT_LINEAR_TET)
    xp, vp = b.device_state()
    p = ctypes.c_void_p
    st = _lib.load().gbfem_adjoint_step(b.handle, 1e-3, p(xp), p(vp), p(vp), p(xp), p(vp), p(xp), p(vp), None, None, 0)
    assert st == _lib.GBFEM_INVALID_ARG
