"""The compression bar over its whole run against the oracle, including the hold phase where
elements invert, and the corotational element's early return for a singular G on a collapsed
element.

The bar is the 40x40x160 benchmark scene reduced to 6x6x24 cubes (4,320 tets, h = 4 mm; per-element
E log-uniform in [1e4, 1e6] Pa, nu uniform in [0.40, 0.49]; z = 0 clamped; the far face driven by a
20% compression ramp over 50 steps, then held; 200 steps). On it the oracle sees its first inverted
element at step 52 and one to three inverted elements through the rest of the hold. Inverted
elements take the SVD polar decomposition (the reflection on the smallest singular value,
Fem3DElementCorotationalTetrahedron.cpp:154), which the GPU kernels run as their FP64 fallback."""

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _run_bar(precision, steps=200, every=10):
    """GPU and oracle side by side; per compared step the relative displacement error, and the
    number of inverted elements and GPU polar fallbacks seen."""
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    sc = mesh.scene_bar_compression(a=6, b=6, c=24)
    g = Body.from_scene(sc, precision=precision)
    o = O.OracleModel.from_scene(sc)
    rest = sc.mesh.nodes.ravel()
    errs, inverted, fallbacks = [], 0, 0
    for s in range(steps):
        vals = sc.driven_values(s)
        g.set_velocities(sc.driven_dofs, vals)
        x, v = o.state()
        v[sc.driven_dofs] = vals
        o.set_state(None, v)
        assert g.step(sc.dt, 1) == _lib.GBFEM_OK
        fallbacks += g.stats()["polar_fallbacks"]
        assert o.step(sc.dt) == 0
        if (s + 1) % every == 0 or s + 1 == steps:
            gx, _ = g.state()
            ox, _ = o.state()
            errs.append(rel(gx - rest, ox - rest))
            inverted = max(inverted, int((mesh.signed_volumes(ox.reshape(-1, 3), sc.mesh.tets) <= 0).sum()))
    return np.array(errs), inverted, fallbacks


def test_bar_fp64_whole_run_matches_oracle(gpu_lib):
    errs, inverted, fallbacks = _run_bar(_lib.PRECISION_FP64)
    print(f"fp64 bar: max rel disp err {errs.max():.2e}, final {errs[-1]:.2e}, inverted {inverted}, "
          f"fallbacks {fallbacks}")
    assert inverted > 0 and fallbacks > 0  # the hold phase exercises the SVD path
    assert errs.max() <= 1e-8


def test_bar_mixed_whole_run_matches_oracle(gpu_lib):
    errs, inverted, fallbacks = _run_bar(_lib.PRECISION_MIXED)
    print(f"mixed bar: max rel disp err {errs.max():.2e}, final {errs[-1]:.2e}, inverted {inverted}, "
          f"fallbacks {fallbacks}")
    assert inverted > 0 and fallbacks > 0
    assert errs.max() <= 1e-6


@pytest.mark.parametrize("precision", [_lib.PRECISION_FP64, _lib.PRECISION_MIXED])
def test_collapsed_element_takes_the_singular_g_return(gpu_lib, precision):
    """A tetrahedron whose nodes lie on one line has a rank-1 deformation gradient, so
    G = (tr(S) I - S) R^T is singular and the reference skips the element's dR/dx terms
    (Fem3DElementCorotationalTetrahedron.cpp:208-216) and goes on with the step. One tetrahedron
    (its node 0 fixed) collapsed onto a line, stepped once on the GPU: both forms take the early
    return exactly where the oracle does, and the step stays finite. The state after it is not
    compared: the polar rotation of a rank-1 F is not unique (any completion of its singular vectors
    is one), so the reference's own result there depends on its SVD's choices; the early return's K
    and force are pinned element by element in tests/test_element_math.py."""
    from oracle import oracle as O
    from opensurgsim_gb300.body import Body

    h = 0.01
    nodes = np.array([[0, 0, 0], [h, 0, 0], [0, h, 0], [0, 0, h]], dtype=np.float64)
    m = mesh.TetMesh(nodes, np.array([[0, 1, 2, 3]], dtype=np.int32), np.array([1e5]), np.array([0.45]),
                     np.array([1000.0]), np.arange(3, dtype=np.int32), (1, 1, 1), h)
    d = np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])
    x = np.stack([t * d for t in (0.0, 0.004, 0.007, 0.011)])  # node 0 stays at the origin
    kw = dict(rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0.0, 0.0, -9.81), cg_tolerance=1e-12)
    g = Body(m, precision=precision, **kw)
    o = O.OracleModel(m, **kw)
    g.set_state(x.ravel(), None)
    o.set_state(x.ravel(), None)
    assert g.step(1e-3, 1) == _lib.GBFEM_OK
    assert o.step(1e-3) == 0
    assert g.stats()["singular_g"] == 1
    assert o.last_stats.singular_g == 1
    gx, gv = g.state()
    assert np.all(np.isfinite(gx)) and np.all(np.isfinite(gv))
