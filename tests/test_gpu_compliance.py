"""Compliance on the GPU (gbfem_apply_compliance, the multi-right-hand-side CG) against the oracle's
applyCompliance, with and without compliance warping."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _pair(precision, tol=1e-12, steps=4, seed=3):
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(3, 4, 5, seed=seed, young=3e5)
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=tol)
    b = Body(s.mesh, precision=precision, **kw)
    o = O.OracleModel(s.mesh, **kw)
    rng = np.random.default_rng(seed)
    # A rotated, moving start so that the element rotations (and the warping) are far from identity.
    c, sn = np.cos(0.4), np.sin(0.4)
    R = np.array([[c, 0.0, sn], [0.0, 1.0, 0.0], [-sn, 0.0, c]])
    x = (R @ s.mesh.nodes.T).T.ravel() + rng.normal(0, 2e-4, 3 * s.mesh.num_nodes)
    v = rng.normal(0, 0.02, x.size)
    b.set_state(x, v)
    o.set_state(x, v)
    for _ in range(steps):
        assert b.step(1e-3) == _lib.GBFEM_OK
        assert o.step(1e-3) == 0
    B = rng.normal(size=(b.n, 11))     # two batches of columns (8 + 3)
    return s, b, o, B


@pytest.mark.parametrize("warping", [False, True])
def test_fp64_compliance_matches_oracle(gpu_lib, warping):
    s, b, o, B = _pair(_lib.PRECISION_FP64)
    X, st, it = b.apply_compliance(B, warping=warping)
    OX, ost, oit = o.apply_compliance(B, warping=warping)
    assert st == _lib.GBFEM_OK and ost == 0
    assert rel(X, OX) <= 1e-8
    assert np.all(X[s.mesh.bc_dofs] == 0.0) or warping
    assert abs(it - oit) <= 0.05 * oit + 11


def test_mixed_compliance_matches_oracle(gpu_lib):
    s, b, o, B = _pair(_lib.PRECISION_MIXED, tol=1e-10)
    X, st, _ = b.apply_compliance(B)
    OX, _, _ = o.apply_compliance(B)
    assert st == _lib.GBFEM_OK
    assert rel(X, OX) <= 1e-5


def test_compliance_columns_are_independent_and_repeatable(gpu_lib):
    s, b, o, B = _pair(_lib.PRECISION_FP64)
    X1, _, _ = b.apply_compliance(B)
    X2, _, _ = b.apply_compliance(B[:, 3:5])
    X3, _, _ = b.apply_compliance(B)
    assert np.array_equal(X1, X3)
    assert rel(X2, X1[:, 3:5]) <= 1e-12


def test_compliance_needs_a_step(gpu_lib):
    from opensurgsim_gb300.body import Body

    s = mesh.scene_cube(2, 2, 2)
    b = Body(s.mesh)
    with pytest.raises(_lib.GbfemError):
        b.apply_compliance(np.ones((b.n, 1)))
