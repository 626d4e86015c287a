"""Hexahedral path (Fem3DElementCube stepped by OdeSolverEulerImplicit) on the GPU against the
oracle's Fem3DElementCube."""

import ctypes

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu

HEX = _lib.ELEMENT_HEXAHEDRON
KW = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _moving_start(s, seed):
    rng = np.random.default_rng(seed)
    x = s.mesh.nodes.ravel() + rng.normal(0, 2e-4, 3 * s.mesh.num_nodes)
    v = rng.normal(0, 0.02, 3 * s.mesh.num_nodes)
    x[s.mesh.bc_dofs] = s.mesh.nodes.ravel()[s.mesh.bc_dofs]
    v[s.mesh.bc_dofs] = 0.0
    return x, v


def _pair(precision, steps=30, seed=2, tol=1e-12, dims=(4, 3, 5), **over):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(*dims, seed=seed, jitter=0.1, young=2e5, poisson=0.42)
    kw = dict(KW, cg_tolerance=tol, **over)
    b = Body(s.mesh, precision=precision, element_type=HEX, **kw)
    o = O.OracleModel(s.mesh, element_type=2, **kw)
    x, v = _moving_start(s, seed)
    b.set_state(x, v)
    o.set_state(x, v)
    launches = []
    for _ in range(steps):
        assert b.step(1e-3) == _lib.GBFEM_OK
        launches.append(b.stats()["kernel_launches"])
        assert o.step(1e-3) == 0
    return s, b, o, launches


def test_hex_fp64_matches_oracle_and_reuses_the_system(gpu_lib):
    s, b, o, launches = _pair(_lib.PRECISION_FP64)
    x, v = b.state()
    ox, ov = o.state()
    x0 = s.mesh.nodes.ravel()
    assert rel(x - x0, ox - x0) <= 1e-8
    assert rel(v, ov) <= 1e-8
    # The first step forms S; later steps run the right-hand side and the solve only.
    assert launches[0] == launches[1] + 1 and all(l == launches[1] for l in launches[2:])


def test_hex_mixed_matches_oracle(gpu_lib):
    s, b, o, launches = _pair(_lib.PRECISION_MIXED, tol=1e-10)
    x, _ = b.state()
    ox, _ = o.state()
    x0 = s.mesh.nodes.ravel()
    assert rel(x - x0, ox - x0) <= 1e-6
    assert launches[0] == launches[1] + 1


def test_hex_newton_iterations_match_oracle(gpu_lib):
    s, b, o, _ = _pair(_lib.PRECISION_FP64, steps=6, newton_max_iterations=3, newton_epsilon=1e-12)
    x0 = s.mesh.nodes.ravel()
    assert rel(b.state()[0] - x0, o.state()[0] - x0) <= 1e-8


def test_divisible_cube_scene_matches_oracle(gpu_lib):
    """The reference's performance-test cube (nu = 0.499, CG tolerance 1e-3, maxIter 0.1 n): same CG
    iteration counts and states as the oracle over its 10 frames."""
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_divisible_cube(6)
    kw = dict(rayleigh_mass=s.rayleigh_mass, rayleigh_stiffness=s.rayleigh_stiffness, gravity=s.gravity,
              cg_tolerance=s.cg_tolerance, cg_max_iterations=s.cg_max_iterations)
    b = Body(s.mesh, element_type=HEX, **kw)
    o = O.OracleModel(s.mesh, element_type=2, **kw)
    for _ in range(s.steps):
        st = b.step(s.dt)
        ost = o.step(s.dt)
        assert st in (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER) and (st == _lib.GBFEM_OK) == (ost == 0)
        assert abs(b.stats()["cg_iterations"] - o.last_stats.cg_iterations) <= 1
    x0 = s.mesh.nodes.ravel()
    assert rel(b.state()[0] - x0, o.state()[0] - x0) <= 1e-6


def test_hex_graph_steps_equal_regular_steps(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(4, 3, 5, seed=7, jitter=0.1)
    kw = dict(KW, cg_tolerance=1e-10, precision=_lib.PRECISION_MIXED, element_type=HEX)
    a = Body(s.mesh, **kw)
    g = Body(s.mesh, **kw)
    g.set_tuning(*a.tuning())
    x, v = _moving_start(s, 7)
    a.set_state(x, v)
    g.set_state(x, v)
    assert a.step(1e-3, 6) == _lib.GBFEM_OK
    assert g.step(1e-3, 6, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    assert np.array_equal(a.state()[0], g.state()[0])


def test_hex_autotune_then_graph(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(6, 6, 8, seed=3, jitter=0.1)
    b = Body(s.mesh, precision=_lib.PRECISION_MIXED, element_type=HEX, autotune=True, cg_tolerance=1e-10, **KW)
    assert b.step(1e-3, 5, _lib.STEP_GRAPH) == _lib.GBFEM_OK
    e, c, r, g = b.tuning()
    assert c in (2, 3, 4) and r in (1, 2, 3, 4)
    assert np.all(np.isfinite(b.state()[0]))


def test_hex_material_change_rebuilds_the_operators(gpu_lib):
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(3, 3, 4, seed=6, jitter=0.1, young=1e5)
    kw = dict(KW, cg_tolerance=1e-12, element_type=HEX)
    a = Body(s.mesh, **kw)
    assert a.step(1e-3, 3) == _lib.GBFEM_OK
    x, v = a.state()
    E2 = torch.full((s.mesh.num_tets,), 3e5, dtype=torch.float64, device="cuda:0")
    nu2 = torch.full((s.mesh.num_tets,), 0.3, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    assert _lib.load().gbfem_set_materials_device(a.handle, ctypes.c_void_p(E2.data_ptr()),
                                                  ctypes.c_void_p(nu2.data_ptr())) == 0
    s2 = mesh.scene_hex_cube(3, 3, 4, seed=6, jitter=0.1, young=3e5, poisson=0.3)
    b = Body(s2.mesh, **kw)
    b.set_state(x, v)
    assert a.step(1e-3, 2) == _lib.GBFEM_OK
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    x0 = s.mesh.nodes.ravel()
    assert rel(a.state()[0] - x0, b.state()[0] - x0) <= 1e-12


def test_hex_dt_change_reforms_the_system(gpu_lib):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(3, 4, 4, seed=9, jitter=0.1)
    kw = dict(KW, cg_tolerance=1e-12)
    b = Body(s.mesh, element_type=HEX, **kw)
    o = O.OracleModel(s.mesh, element_type=2, **kw)
    for dt in (1e-3, 1e-3, 2e-3, 5e-4, 5e-4):
        assert b.step(dt) == _lib.GBFEM_OK
        assert o.step(dt) == 0
    x0 = s.mesh.nodes.ravel()
    assert rel(b.state()[0] - x0, o.state()[0] - x0) <= 1e-8


def test_hex_batch_matches_single_meshes(gpu_lib):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    scenes = [mesh.scene_hex_cube(*d, seed=k, jitter=0.1, young=10 ** (4 + k)) for k, d in
              enumerate([(2, 2, 3), (4, 3, 3), (3, 5, 2)])]
    kw = dict(KW, cg_tolerance=1e-10)
    b = Body([sc.mesh for sc in scenes], precision=_lib.PRECISION_MIXED, element_type=HEX, **kw)
    assert b.step(1e-3, 10) == _lib.GBFEM_OK
    x, _ = b.state()
    for k, sc in enumerate(scenes):
        o = O.OracleModel(sc.mesh, element_type=2, **kw)
        assert o.step(1e-3, 10) == 0
        n0, n1 = 3 * b.node_offsets[k], 3 * b.node_offsets[k + 1]
        x0 = sc.mesh.nodes.ravel()
        assert rel(x[n0:n1] - x0, o.state()[0] - x0) <= 1e-6


def test_hex_compliance_matches_oracle(gpu_lib):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(3, 3, 4, seed=4, jitter=0.1)
    kw = dict(KW, cg_tolerance=1e-12)
    b = Body(s.mesh, element_type=HEX, **kw)
    o = O.OracleModel(s.mesh, element_type=2, **kw)
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    assert o.step(1e-3, 2) == 0
    B = np.random.default_rng(0).normal(size=(b.n, 5))
    X, st, _ = b.apply_compliance(B)
    OX, ost, _ = o.apply_compliance(B)
    assert st == _lib.GBFEM_OK and ost == 0
    assert rel(X, OX) <= 1e-8
    with pytest.raises(_lib.GbfemError):
        b.apply_compliance(B, warping=True)


def test_hex_rejects_tetrahedron_only_features(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_hex_cube(2, 2, 2)
    b = Body(s.mesh, element_type=HEX)
    with pytest.raises(_lib.GbfemError):
        b.step(1e-3, 1, _lib.STEP_KEEP_SYSTEM)
    xp, vp = b.device_state()
    p = ctypes.c_void_p
    st = _lib.load().gbfem_adjoint_step(b.handle, 1e-3, p(xp), p(vp), p(vp), p(xp), p(vp), p(xp), p(vp), None, None, 0)
    assert st == _lib.GBFEM_INVALID_ARG
    # The element-to-nonzero map covers 24 x 24 entries per hexahedron and matches the oracle's.
    from oracle import oracle as O

    o = O.OracleModel(s.mesh, element_type=2)
    assert np.array_equal(b.scatter(), o.scatter())
