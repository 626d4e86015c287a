"""The oracle's Fem3DElementCube (hexahedron) against the known answers of the reference's own
element tests (Fem3DElementCubeTests.cpp) and an independent numpy derivation.

Known answers restated here:
  * SetUp (:425-478): a unit cube centred on the origin, element node ids {0,1,3,2,4,5,7,6} over the
    corners listed there; rho = 1000, E = 1e6, nu = 0.45; rest volume 1.
  * computeExpectedStiffnessMatrix (:102-372): the closed-form stiffness of the unit cube with
    a = E(1-nu)/((1+nu)(1-2nu)), b = E nu/((1+nu)(1-2nu)), c = E/(2(1+nu)) (Muller, Teschner, Gross,
    CGI 2004, with the diagonal of block (4,4) corrected to d as the test notes).
  * computeExpectedMassMatrix (:374-423): rho/27 on the diagonal, halved per coordinate in which
    the two corners differ.
  * VolumeTest (:561-588), NodeOrderingTest (:590-648), ShapeFunctionsTest (:650-795),
    ForceAndMatricesTest (:865-953: no force at rest).
"""

import itertools

import numpy as np
import pytest

from oracle import oracle as O

# The reference test's 8 cube points (:441-448) and its element node ids (:453).
POINTS = np.array([[-0.5, -0.5, -0.5], [0.5, -0.5, -0.5], [-0.5, 0.5, -0.5], [0.5, 0.5, -0.5],
                   [-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [-0.5, 0.5, 0.5], [0.5, 0.5, 0.5]])
NODE_IDS = [0, 1, 3, 2, 4, 5, 7, 6]
RHO, YOUNG, NU = 1000.0, 1e6, 0.45
SIGNS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)


def _x0(ids):
    return POINTS[list(ids)].ravel()


def _independent_k_m(x0, E, nu, rho):
    """K and M of a trilinear hexahedron by a 3-point Gauss rule (exact for the unit cube, where the
    integrands are at most quadratic per coordinate) and the closed-form block
    K_ab(i,j) = lam g_a,i g_b,j + mu g_a,j g_b,i + mu delta_ij (g_a . g_b)."""
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    pts, wts = np.polynomial.legendre.leggauss(3)
    p = x0.reshape(8, 3)
    K = np.zeros((24, 24))
    M = np.zeros((24, 24))
    for (e, we), (h, wh), (m, wm) in itertools.product(zip(pts, wts), repeat=3):
        xi = np.array([e, h, m])
        one = 1 + SIGNS * xi                       # (8, 3)
        N = one.prod(axis=1) / 8
        dN = np.stack([SIGNS[:, 0] * one[:, 1] * one[:, 2], one[:, 0] * SIGNS[:, 1] * one[:, 2],
                       one[:, 0] * one[:, 1] * SIGNS[:, 2]], axis=1) / 8    # (8, 3) natural
        J = dN.T @ p                                # J[r, axis]
        g = np.linalg.solve(J, dN.T).T              # (8, 3) spatial gradients
        w = we * wh * wm * np.linalg.det(J)
        for a in range(8):
            for b in range(8):
                blk = lam * np.outer(g[a], g[b]) + mu * np.outer(g[b], g[a]) + mu * (g[a] @ g[b]) * np.eye(3)
                K[3 * a:3 * a + 3, 3 * b:3 * b + 3] += w * blk
                M[3 * a:3 * a + 3, 3 * b:3 * b + 3] += w * rho * N[a] * N[b] * np.eye(3)
    return K, M


def test_unit_cube_stiffness_and_mass_match_the_independent_derivation():
    r = O.hex_compute(_x0(NODE_IDS), None, YOUNG, NU, RHO)
    K, M = _independent_k_m(_x0(NODE_IDS), YOUNG, NU, RHO)
    assert abs(r["volume"] - 1.0) <= 1e-10
    assert np.allclose(r["K"], K, rtol=0, atol=1e-9 * np.abs(K).max())
    assert np.allclose(r["M"], M, rtol=0, atol=1e-12 * np.abs(M).max())


def test_unit_cube_stiffness_matches_the_published_closed_form():
    K = O.hex_compute(_x0(NODE_IDS), None, YOUNG, NU, RHO)["K"]
    a = YOUNG * (1 - NU) / ((1 + NU) * (1 - 2 * NU))
    b = YOUNG * NU / ((1 + NU) * (1 - 2 * NU))
    c = YOUNG / (2 * (1 + NU))
    blk = lambda i, j: K[3 * i:3 * i + 3, 3 * j:3 * j + 3]
    tol = 1e-9 * a
    # Diagonal block of corner 0: d on the diagonal, e elsewhere.
    d, e = (a + 2 * c) / 9, (b + c) / 12
    assert np.allclose(blk(0, 0), np.full((3, 3), e) + (d - e) * np.eye(3), atol=tol)
    # Corner 4's diagonal block: d on the whole diagonal (the corrected entry), e at (0,1)/(1,0), -e else.
    exp = np.full((3, 3), -e)
    np.fill_diagonal(exp, d)
    exp[0, 1] = exp[1, 0] = e
    assert np.allclose(blk(4, 4), exp, atol=tol)
    # Edge along x, corners 0-1.
    d1, d2, e1, e2 = (-a + c) / 9, (a - c) / 18, (b - c) / 12, (b + c) / 24
    assert np.allclose(blk(0, 1), [[d1, e1, e1], [-e1, d2, e2], [-e1, e2, d2]], atol=tol)
    # Face diagonal, corners 0-2.
    fd1, fd2, fe1, fe2 = (-2 * a - c) / 36, (a - 4 * c) / 36, (b + c) / 12, (b - c) / 24
    assert np.allclose(blk(0, 2), [[fd1, -fe1, fe2], [-fe1, fd1, fe2], [-fe2, -fe2, fd2]], atol=tol)
    # Body diagonal, corners 0-6.
    bd, be = (-a - 2 * c) / 36, (b + c) / 24
    assert np.allclose(blk(0, 6), np.full((3, 3), -be) + (bd + be) * np.eye(3), atol=tol)


def test_unit_cube_mass_matches_the_closed_form():
    M = O.hex_compute(_x0(NODE_IDS), None, YOUNG, NU, RHO)["M"]
    for i in range(8):
        for j in range(8):
            differ = int(np.sum(SIGNS[i] != SIGNS[j]))
            assert np.allclose(M[3 * i:3 * i + 3, 3 * j:3 * j + 3], RHO / 27 / 2 ** differ * np.eye(3), atol=1e-9)


def test_no_force_at_rest_and_linear_force():
    x0 = _x0(NODE_IDS)
    r = O.hex_compute(x0, x0, YOUNG, NU, RHO)
    assert np.all(r["f"] == 0.0)
    u = np.random.default_rng(0).normal(0, 1e-3, 24)
    r = O.hex_compute(x0, x0 + u, YOUNG, NU, RHO)
    assert np.allclose(r["f"], -r["K"] @ u, rtol=1e-12, atol=1e-12 * np.abs(r["f"]).max())


def test_distorted_hexahedron_rigid_modes_and_spectrum():
    rng = np.random.default_rng(4)
    x0 = (SIGNS * 0.5 + rng.uniform(-0.08, 0.08, (8, 3))).ravel()
    r = O.hex_compute(x0, None, 2e5, 0.3, 1100.0)
    K, M = r["K"], r["M"]
    Ki, Mi = _independent_k_m(x0, 2e5, 0.3, 1100.0)
    # Distorted: 2x2x2 Gauss is no longer exact, so the 3-point derivation differs; the oracle must
    # still be symmetric, annihilate rigid motions, and have exactly six zero eigenvalues.
    assert np.allclose(K, K.T, atol=1e-10 * np.abs(K).max())
    p = x0.reshape(8, 3)
    for axis in range(3):
        t = np.zeros((8, 3))
        t[:, axis] = 1.0
        assert np.abs(K @ t.ravel()).max() <= 1e-9 * np.abs(K).max()
        w = np.zeros(3)
        w[axis] = 1.0
        assert np.abs(K @ np.cross(w, p).ravel()).max() <= 1e-9 * np.abs(K).max()
    ev = np.linalg.eigvalsh(0.5 * (K + K.T))
    assert np.sum(np.abs(ev) < 1e-9 * ev.max()) == 6 and ev.min() > -1e-9 * ev.max()
    assert np.allclose(M.sum(), 3 * 1100.0 * r["volume"])
    assert np.allclose(np.linalg.eigvalsh(M).min() > 0, True)
    assert np.abs(K - Ki).max() <= 0.2 * np.abs(K).max()   # same operator, different quadrature


def test_volume_and_invalid_elements():
    assert abs(O.hex_compute(_x0(NODE_IDS), None, YOUNG, NU, RHO)["volume"] - 1.0) <= 1e-10
    with pytest.raises(O.OracleError):                       # valid but negative volume
        O.hex_compute(_x0([0, 1, 3, 2, 4, 6, 7, 5]), None, YOUNG, NU, RHO)
    flat = POINTS.copy()
    flat[4:] = flat[:4]                                      # cube degenerated to a square
    with pytest.raises(O.OracleError):
        O.hex_compute(flat[NODE_IDS].ravel(), None, YOUNG, NU, RHO)
    for bad in [(0.0, NU, RHO), (YOUNG, 0.5, RHO), (YOUNG, NU, -1.0)]:
        with pytest.raises(O.OracleError):
            O.hex_compute(_x0(NODE_IDS), None, *bad)


# (first face, opposite face, expect failure) of NodeOrderingTest, every rotation of either face.
ORDERINGS = [
    ((6, 7, 5, 4), (2, 3, 1, 0), False), ((6, 7, 5, 4), (2, 0, 1, 3), True),
    ((6, 4, 5, 7), (2, 3, 1, 0), True), ((6, 4, 5, 7), (2, 0, 1, 3), True),
    ((0, 1, 3, 2), (4, 5, 7, 6), False), ((0, 1, 3, 2), (4, 6, 7, 5), True),
    ((0, 2, 3, 1), (4, 5, 7, 6), True), ((0, 2, 3, 1), (4, 6, 7, 5), True),
    ((2, 3, 7, 6), (0, 1, 5, 4), False), ((2, 3, 7, 6), (0, 4, 5, 1), True),
    ((2, 6, 7, 3), (0, 1, 5, 4), True), ((2, 6, 7, 3), (0, 4, 5, 1), True),
    ((0, 4, 5, 1), (6, 7, 3, 2), False), ((0, 4, 5, 1), (6, 2, 3, 7), True),
    ((0, 1, 5, 4), (6, 7, 3, 2), True), ((0, 1, 5, 4), (6, 2, 3, 7), True),
    ((3, 1, 5, 7), (2, 0, 4, 6), False), ((3, 1, 5, 7), (2, 6, 4, 0), True),
    ((3, 7, 5, 1), (2, 0, 4, 6), True), ((3, 7, 5, 1), (2, 6, 4, 0), True),
    ((0, 2, 6, 4), (1, 3, 7, 5), False), ((0, 2, 6, 4), (1, 5, 7, 3), True),
    ((0, 4, 6, 2), (1, 3, 7, 5), True), ((0, 4, 6, 2), (1, 5, 7, 3), True),
]


def hex_orderings():
    for f1, f2, bad in ORDERINGS:
        for r1 in range(4):
            for r2 in range(4):
                yield [f1[(i + r1) % 4] for i in range(4)] + [f2[(i + r2) % 4] for i in range(4)], bad


def test_node_orderings_match_the_reference():
    count = 0
    for ids, bad in hex_orderings():
        count += 1
        if bad:
            with pytest.raises(O.OracleError):
                O.hex_compute(_x0(ids), None, YOUNG, NU, RHO)
        else:
            O.hex_compute(_x0(ids), None, YOUNG, NU, RHO)
    assert count == 24 * 16


def test_shape_functions():
    for i in range(8):
        for j in range(8):
            assert abs(O.hex_shape(i, *SIGNS[j])[0] - (1.0 if i == j else 0.0)) <= 1e-12
    grid = np.arange(-1.0, 1.0001, 0.1)
    for e, h, m in itertools.product(grid[::4], grid[::3], grid[::5]):
        vals = np.array([O.hex_shape(i, e, h, m) for i in range(8)])
        assert abs(vals[:, 0].sum() - 1.0) <= 1e-10
        assert np.abs(vals[:, 1:].sum(axis=0)).max() <= 1e-12   # derivatives of a partition of unity


def _dense_step(mesh, x, v, dt, alpha, beta, g):
    """One implicit Euler step of a hexahedral mesh, independently: element K/M from the numpy
    derivation, dense assembly, S = M/dt + D + dt K, BC rows/columns zeroed with unit diagonal,
    rhs = f - dt K v (first Newton iteration), dense solve."""
    n = 3 * mesh.num_nodes
    Kg = np.zeros((n, n))
    Mg = np.zeros((n, n))
    lumped = np.zeros(mesh.num_nodes)
    for e, nd in enumerate(mesh.tets):
        x0 = mesh.nodes[nd].ravel()
        K, M = _independent_k_m(x0, mesh.young[e], mesh.poisson[e], mesh.density[e])
        dofs = (3 * nd[:, None] + np.arange(3)).ravel()
        Kg[np.ix_(dofs, dofs)] += K
        Mg[np.ix_(dofs, dofs)] += M
        lumped[nd] += M[0::3, 0::3].sum() / 8      # rho V / 8 (the scalar mass blocks sum to rho V)
    x0 = mesh.nodes.ravel()
    f = -Kg @ (x - x0) - (alpha * Mg + beta * Kg) @ v + np.repeat(lumped, 3) * np.tile(g, mesh.num_nodes)
    S = Mg / dt + alpha * Mg + beta * Kg + dt * Kg
    rhs = f - dt * Kg @ v
    for d in mesh.bc_dofs:
        S[d, :] = 0
        S[:, d] = 0
        S[d, d] = 1
        rhs[d] = 0
    dv = np.linalg.solve(S, rhs)
    vn = v + dv
    return x + dt * vn, vn


def test_oracle_hex_step_matches_an_independent_dense_step():
    from opensurgsim_gb300 import mesh as msh

    s = msh.scene_hex_cube(2, 2, 3, h=0.01, young=2e5, poisson=0.4, density=1000.0)
    kw = dict(rayleigh_mass=0.02, rayleigh_stiffness=0.001, gravity=(0.0, 0.0, -9.81), cg_tolerance=1e-14)
    o = O.OracleModel(s.mesh, element_type=2, **kw)
    rng = np.random.default_rng(1)
    x = s.mesh.nodes.ravel() + rng.normal(0, 1e-4, 3 * s.mesh.num_nodes)
    v = rng.normal(0, 0.01, 3 * s.mesh.num_nodes)
    x[s.mesh.bc_dofs] = s.mesh.nodes.ravel()[s.mesh.bc_dofs]
    v[s.mesh.bc_dofs] = 0.0
    o.set_state(x, v)
    assert o.step(1e-3) == 0
    ox, ov = o.state()
    ex, ev = _dense_step(s.mesh, x, v, 1e-3, 0.02, 0.001, np.array([0.0, 0.0, -9.81]))
    assert np.linalg.norm(ov - ev) <= 1e-9 * np.linalg.norm(ev)
    assert np.linalg.norm(ox - ex) <= 1e-12 * np.linalg.norm(ex)
    # Lumped gravity mass rho V / 8 per node.
    assert np.allclose(o.mass_per_node().sum(), 1000.0 * 2 * 2 * 3 * 1e-6)


def test_divisible_cube_scene():
    from opensurgsim_gb300 import mesh as msh

    s = msh.scene_divisible_cube(4)
    assert s.mesh.num_nodes == 64 and s.mesh.num_tets == 27
    assert np.allclose(s.mesh.nodes.min(axis=0), -4.0) and np.allclose(s.mesh.nodes.max(axis=0), 4.0)
    assert list(s.mesh.bc_dofs) == list(range(9))
    o = O.OracleModel.from_scene(s, element_type=2)
    assert o.mass_per_node().sum() == pytest.approx(980.0 * 8.0 ** 3)
    assert o.step(s.dt, s.steps) in (0, 3)
    x, v = o.state()
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(v))
