"""The oracle's implicit-Euler / CG semantics against the reference's own tests (CPU)."""

import numpy as np
import pytest

from oracle import oracle as O
from opensurgsim_gb300 import mesh


def approx(a, b, prec):
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))


def cg_matrix(n=18):
    # LinearSparseSolveAndInverseTests.cpp:57-88
    r, c = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    A = np.fmod(10.3 * np.cos((r * c).astype(float)) + 3.24, 10.0)
    b = np.fmod(-4.1 * np.arange(n) ** 2 + 3.46, 5.0)
    colptr = np.arange(0, n * n + 1, n, dtype=np.int32)
    rowidx = np.tile(np.arange(n, dtype=np.int32), n)
    return A, b, colptr, rowidx, A.T.ravel().copy()


def test_cg_max_iterations_behaviour():
    """SparseCGMatrixComponentsTest (LinearSparseSolveAndInverseTests.cpp:162-193)."""
    A, b, colptr, rowidx, vals = cg_matrix()
    expected = np.linalg.solve(A, b)
    x, it, err, st = O.cg_solve(colptr, rowidx, vals, b)  # Eigen defaults: tol = eps, maxIter = 2n
    assert approx(x, expected, 1e-5)
    x, it, err, st = O.cg_solve(colptr, rowidx, vals, b, tol=1e-10, max_iter=18)
    assert approx(x, expected, 1e-5) and not approx(x, expected, 1e-10)
    assert st == O.ORC_CG_MAXITER and it == 18
    x, it, err, st = O.cg_solve(colptr, rowidx, vals, b, tol=1e-10, max_iter=50)
    assert approx(x, expected, 1e-10) and st == O.ORC_OK


def test_cg_reads_only_lower_triangle_and_zero_rhs():
    A, b, colptr, rowidx, vals = cg_matrix(6)
    A = A @ A.T + 6 * np.eye(6)  # SPD
    vals = A.T.ravel().copy()
    x_ref, *_ = O.cg_solve(colptr, rowidx, vals, b, tol=1e-14)
    junk = vals.copy().reshape(6, 6)  # column-major: junk[c, r] = A[r, c]
    for c in range(6):
        for r in range(c):
            junk[c, r] = 1e6  # upper triangle entries (r < c) must be ignored
    x, *_ = O.cg_solve(colptr, rowidx, junk.ravel(), b, tol=1e-14)
    assert np.allclose(x, x_ref, rtol=1e-12, atol=1e-14)
    x, it, err, st = O.cg_solve(colptr, rowidx, vals, np.zeros(6), tol=1e-10)
    assert np.all(x == 0) and it == 0 and st == O.ORC_OK


@pytest.mark.parametrize("visc", [0.0, 0.1])
def test_mass_point_backward_euler(visc):
    """OdeSolverEulerImplicitTests.cpp:58-115 (MassPoint, mass 0.456, gravity (0,-9.81,0))."""
    dt, m, g = 1e-3, 0.456, np.array([0.0, -9.81, 0.0])
    x0, v0 = np.zeros(3), np.zeros(3)
    x1, v1 = O.masspoint_step(visc, dt, x0, v0)
    expected_v = (g * dt + v0) / (1.0 + dt * visc / m)
    assert np.allclose(v1, expected_v, rtol=1e-12, atol=1e-15)
    assert np.allclose(x1, v1 * dt + x0, rtol=1e-12, atol=1e-15)
    x2, v2 = O.masspoint_step(visc, dt, x1, v1)
    assert np.allclose(v2, (g * dt + v1) / (1.0 + dt * visc / m), rtol=1e-12)


def test_free_fall_uniform_velocity():
    """No boundary conditions: K annihilates translations and the consistent mass has lumped row
    sums, so the first step is a uniform velocity g dt / (1 + alpha dt)."""
    s = mesh.scene_cube(3, 3, 3)
    s.mesh.bc_dofs = np.zeros(0, dtype=np.int32)
    m = O.OracleModel(s.mesh, rayleigh_mass=0.01, rayleigh_stiffness=0.001, gravity=(0, 0, -9.81), cg_tolerance=1e-14)
    assert m.step(1e-3) == O.ORC_OK
    x, v = m.state()
    expected = -9.81 * 1e-3 / (1 + 0.01 * 1e-3)
    assert np.allclose(v.reshape(-1, 3)[:, 2], expected, rtol=1e-9)
    assert np.allclose(v.reshape(-1, 3)[:, :2], 0, atol=1e-12)


def test_rigid_rotation_has_no_elastic_force():
    s = mesh.scene_cube(2, 2, 2)
    m = O.OracleModel(s.mesh, gravity_enabled=False, cg_tolerance=1e-14)
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    x = (R @ s.mesh.nodes.T).T.ravel() + 0.3
    m.set_state(x, np.zeros_like(x))
    m.step(1e-3)
    f = m.system()["f"]
    assert np.abs(f).max() < 1e-9 * s.mesh.young[0] * 0.01


def test_boundary_conditions_and_pattern():
    s = mesh.scene_cube(3, 2, 4)
    m = O.OracleModel.from_scene(s)
    assert m.step(s.dt, 3) == O.ORC_OK
    x, v = m.state()
    bc = s.mesh.bc_dofs
    assert np.array_equal(x[bc], s.mesh.nodes.ravel()[bc]) and np.all(v[bc] == 0)
    colptr, rowidx = m.pattern()
    sy = m.system()
    S = np.zeros((m.n, m.n))
    for c in range(m.n):
        rows = rowidx[colptr[c]:colptr[c + 1]]
        assert np.all(np.diff(rows) > 0)  # sorted, unique
        S[rows, c] = sy["S"][colptr[c]:colptr[c + 1]]
    P = np.zeros_like(S, dtype=bool)
    for c in range(m.n):
        P[rowidx[colptr[c]:colptr[c + 1]], c] = True
    assert np.array_equal(P, P.T)  # structurally symmetric pattern
    for d in bc:  # OdeState::applyBoundaryConditionsToMatrix: zero row/column, diagonal 1
        row = S[d].copy()
        row[d] = 0
        assert np.all(row == 0) and np.all(S[:, d][np.arange(m.n) != d] == 0) and S[d, d] == 1.0
    assert np.all(sy["rhs"][bc] == 0)


def test_nonfinite_state_deactivates():
    s = mesh.scene_cube(2, 2, 2)
    m = O.OracleModel.from_scene(s)
    x, v = m.state()
    v[4] = np.nan
    m.set_state(None, v)
    assert m.step(1e-3) == O.ORC_NONFINITE
    assert m.step(1e-3) == O.ORC_NONFINITE


def test_scatter_map_points_at_block_entries():
    s = mesh.scene_cube(2, 2, 2)
    m = O.OracleModel.from_scene(s)
    colptr, rowidx = m.pattern()
    sc = m.scatter().reshape(-1, 12, 12)
    tets = s.mesh.tets
    for e in range(tets.shape[0]):
        for a in range(4):
            for i in range(3):
                for b in range(4):
                    for j in range(3):
                        k = sc[e, 3 * a + i, 3 * b + j]
                        col = 3 * tets[e, b] + j
                        assert colptr[col] <= k < colptr[col + 1] and rowidx[k] == 3 * tets[e, a] + i


def _csc_matvec(colptr, rowidx, vals, v):
    out = np.zeros_like(v)
    for c in range(len(colptr) - 1):
        sl = slice(colptr[c], colptr[c + 1])
        out[rowidx[sl]] += vals[sl] * v[c]
    return out


def test_linear_tetrahedron_force_and_constant_stiffness():
    """Fem3DElementTetrahedron::doUpdateFMDK (Fem3DElementTetrahedron.cpp:77-90): K does not depend on
    the state and f = -K (x - x0) + gravity - alpha M v - beta K v (FemRepresentation.cpp:479-545)."""
    s = mesh.scene_cube(2, 2, 3)
    alpha, beta = 0.01, 0.001
    m = O.OracleModel(s.mesh, rayleigh_mass=alpha, rayleigh_stiffness=beta, gravity=(0, 0, -9.81),
                      cg_tolerance=1e-14, element_type=1)
    colptr, rowidx = m.pattern()
    rng = np.random.default_rng(4)
    x0 = s.mesh.nodes.ravel()
    Ks = []
    for trial in range(2):
        R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]]) if trial else np.eye(3)
        x = (R @ s.mesh.nodes.T).T.ravel() + rng.normal(0, 1e-4, x0.size)
        v = rng.normal(0, 0.01, x0.size)
        m.set_state(x, v)
        m.step(1e-3)
        sys_ = m.system()
        Ks.append(sys_["K"].copy())
        K, M = sys_["K"], sys_["M"]
        g = np.zeros_like(x0)
        g[2::3] = -9.81 * m.mass_per_node()
        expect = (-_csc_matvec(colptr, rowidx, K, x - x0) + g - alpha * _csc_matvec(colptr, rowidx, M, v)
                  - beta * _csc_matvec(colptr, rowidx, K, v))
        assert np.linalg.norm(sys_["f"] - expect) <= 1e-10 * np.linalg.norm(expect)
    assert np.array_equal(Ks[0], Ks[1])
    # A rigid rotation is not force-free for the linear element (it is for the corotational one).
    assert np.abs(sys_["f"] - g).max() > 1e-3


def _dense(colptr, rowidx, vals, n):
    A = np.zeros((n, n))
    for c in range(n):
        for k in range(colptr[c], colptr[c + 1]):
            A[rowidx[k], c] = vals[k]
    return A


def test_apply_compliance_solves_the_last_system_with_bc_rows_zeroed():
    """DeformableRepresentation::applyCompliance (DeformableRepresentation.cpp:175-191)."""
    s = mesh.scene_cube(2, 2, 2)
    m = O.OracleModel(s.mesh, rayleigh_mass=0.01, rayleigh_stiffness=0.001, cg_tolerance=1e-14)
    m.step(1e-3)
    colptr, rowidx = m.pattern()
    S = _dense(colptr, rowidx, m.system()["S"], m.n)
    S = np.tril(S) + np.tril(S, -1).T      # the CG reads the lower triangle
    B = np.random.default_rng(1).normal(size=(m.n, 3))
    X, st, it = m.apply_compliance(B)
    assert st == 0 and it > 0
    bc = s.mesh.bc_dofs
    Bz = B.copy()
    Bz[bc] = 0
    ref = np.linalg.solve(S, Bz)
    ref[bc] = 0
    assert np.linalg.norm(X - ref) <= 1e-9 * np.linalg.norm(ref)


def test_compliance_warping_uses_the_node_rotations():
    """FemRepresentation::applyCompliance with warping: for a rigidly rotated body every element (and so
    every node) has the body's rotation R, and x = (I (x) R) S^-1 (I (x) R^T) b."""
    s = mesh.scene_cube(2, 2, 2)
    m = O.OracleModel(s.mesh, gravity_enabled=False, cg_tolerance=1e-14)
    c, sn = np.cos(0.6), np.sin(0.6)
    R = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]]) @ np.array([[1.0, 0, 0], [0, c, -sn], [0, sn, c]])
    x = (R @ s.mesh.nodes.T).T.ravel()
    m.set_state(x, np.zeros_like(x))
    m.step(1e-3)
    B = np.random.default_rng(2).normal(size=(m.n, 2))
    Xw, st, _ = m.apply_compliance(B, warping=True)
    assert st == 0
    W = np.kron(np.eye(m.n // 3), R)
    X0, _, _ = m.apply_compliance(W.T @ B)
    assert np.linalg.norm(Xw - W @ X0) <= 1e-10 * np.linalg.norm(Xw)


@pytest.mark.parametrize("gravity,damping", [(False, False), (False, True), (True, False), (True, True)])
def test_fmdk_gravity_damping_and_external_force(gravity, damping):
    """FemRepresentationTests.cpp:236-410 restated on a real mesh, with an external generalized force
    (Fem3DRepresentation.cpp:133-197, applied by FemRepresentation.cpp:527-544):
    f = sum f_e [+ m_node g] [- alpha M v - beta K v] + F_ext, D = [alpha M + beta K] + D_ext,
    K = sum K_e + K_ext, M = sum M_e."""
    import scipy.sparse as sp

    s = mesh.scene_cube(2, 2, 2, seed=3)
    a, b = (0.02, 0.003) if damping else (0.0, 0.0)
    g = np.array([0.0, -9.81, 0.0])
    base = O.OracleModel(s.mesh, gravity_enabled=False, cg_tolerance=1e-14)
    m = O.OracleModel(s.mesh, rayleigh_mass=a, rayleigh_stiffness=b, gravity=tuple(g), gravity_enabled=gravity,
                      cg_tolerance=1e-14)
    rng = np.random.default_rng(11)
    x = s.mesh.nodes.ravel() + rng.normal(0, 1e-4, 3 * s.mesh.num_nodes)
    v = rng.normal(0, 0.05, x.size)
    for mod in (base, m):
        mod.set_state(x, v)
    e = 7
    coord = np.array([0.1, 0.2, 0.3, 0.4])
    F = np.array([1.5, -2.0, 0.5])
    Kx = rng.normal(size=(3, 3))
    Dx = rng.normal(size=(3, 3))
    m.add_external_force(e, coord, F, Kx, Dx)
    assert base.step(1e-3) == 0 and m.step(1e-3) == 0
    colptr, rowidx = m.pattern()
    n = m.n
    sb, sm = base.system(), m.system()
    mat = lambda vals: sp.csc_matrix((vals, rowidx, colptr), shape=(n, n))
    # External blocks on the pattern, from the scatter map of element e.
    kext = np.zeros(m.nnz)
    dext = np.zeros(m.nnz)
    fext = np.zeros(n)
    nd = s.mesh.tets[e]
    slots = m.scatter().reshape(-1, 12, 12)[e]
    for aa in range(4):
        fext[3 * nd[aa]:3 * nd[aa] + 3] += coord[aa] * F
        for bb in range(4):
            kext[slots[3 * aa:3 * aa + 3, 3 * bb:3 * bb + 3].ravel()] += coord[aa] * coord[bb] * Kx.ravel()
            dext[slots[3 * aa:3 * aa + 3, 3 * bb:3 * bb + 3].ravel()] += coord[aa] * coord[bb] * Dx.ravel()
    assert np.allclose(sm["M"], sb["M"], rtol=0, atol=0)
    assert np.allclose(sm["K"], sb["K"] + kext, rtol=1e-14, atol=1e-12 * np.abs(sb["K"]).max())
    assert np.allclose(sm["D"], a * sb["M"] + b * sb["K"] + dext, rtol=1e-14, atol=1e-12 * np.abs(sb["K"]).max())
    want = sb["f"] + fext - a * (mat(sb["M"]) @ v) - b * (mat(sb["K"]) @ v)
    if gravity:
        want += np.repeat(m.mass_per_node(), 3) * np.tile(g, s.mesh.num_nodes)
    assert np.allclose(sm["f"], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    # Cleared after the step (DeformableRepresentation::afterUpdate): the next step has no external load.
    m2 = O.OracleModel(s.mesh, rayleigh_mass=a, rayleigh_stiffness=b, gravity=tuple(g), gravity_enabled=gravity,
                       cg_tolerance=1e-14)
    m2.set_state(*m.state())
    assert m.step(1e-3) == 0 and m2.step(1e-3) == 0
    assert np.array_equal(m.state()[0], m2.state()[0])


@pytest.mark.parametrize("element_type", [0, 2])
def test_mass_lumping(element_type):
    """FemRepresentationTests.cpp:529-572 (MassLumpingTest: after an update with mass lumping on, M
    is diagonal), plus what FemRepresentation.cpp:499-508 and :584-586 imply: every row of the
    lumped M holds the consistent M's row sum on its diagonal (the pattern kept, explicit zeros
    elsewhere); D = alpha M_lumped + beta K; the Rayleigh mass force is alpha diag(M) v; for
    tetrahedra the lumped diagonal is the node's rho V / 4 sum (massPerNode)."""
    import scipy.sparse as sp

    if element_type == 2:
        s = mesh.scene_hex_cube(2, 3, 2, jitter=0.1, seed=4)
    else:
        s = mesh.scene_cube(2, 2, 3, seed=3)
    a, b = 0.02, 0.003
    kw = dict(rayleigh_mass=a, rayleigh_stiffness=b, gravity_enabled=False, cg_tolerance=1e-14,
              element_type=element_type)
    cons = O.OracleModel(s.mesh, **kw)
    lump = O.OracleModel(s.mesh, mass_lumping=True, **kw)
    rng = np.random.default_rng(5)
    x = s.mesh.nodes.ravel() + rng.normal(0, 1e-4, 3 * s.mesh.num_nodes)
    v = rng.normal(0, 0.05, x.size)
    for mod in (cons, lump):
        mod.set_state(x, v)
        assert mod.step(1e-3) == 0
    colptr, rowidx = lump.pattern()
    n = lump.n
    sc, sl = cons.system(), lump.system()
    Mc = sp.csc_matrix((sc["M"], rowidx, colptr), shape=(n, n))
    Ml = sp.csc_matrix((sl["M"], rowidx, colptr), shape=(n, n))
    dense = Ml.toarray()
    assert np.count_nonzero(dense - np.diag(np.diag(dense))) == 0  # isDiagonal()
    assert np.allclose(np.diag(dense), np.asarray(Mc.sum(axis=1)).ravel(), rtol=1e-14, atol=0)
    assert Ml.nnz == Mc.nnz  # zeroRow keeps the pattern
    if element_type == 0:
        assert np.allclose(np.diag(dense), np.repeat(lump.mass_per_node(), 3), rtol=1e-13)
    assert np.allclose(sl["K"], sc["K"], rtol=0, atol=0)
    assert np.allclose(sl["D"], a * sl["M"] + b * sl["K"], rtol=1e-14, atol=1e-14 * np.abs(sl["K"]).max())
    # f differs from the consistent model only in the Rayleigh mass force.
    want = sc["f"] + a * (Mc @ v) - a * np.diag(dense) * v
    assert np.allclose(sl["f"], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_reference_formula_is_translation_variant_in_fp64():
    """The reference's corotational element works on absolute positions (F = P V^-1 with the node
    positions, f = -K (x - R x0), KTimesRx_x0 = K (R^T x - x0); Fem3DElementCorotationalTetrahedron.cpp
    :131-146, :103-113, :276). Translating a strained mesh 10 m (1,000 element sizes) changes nothing
    in exact arithmetic, but the large translation enters those products and cancels only up to FP64
    rounding: the oracle's 3-step displacement moves by about 1e-6 relative (measured 7.5e-7 at CG
    tolerance 1e-12) between the origin and 10 m, 7.4e-9 at 1 m and 2.2e-12 at 1 cm. This is why the
    GPU forms, which work on
    positions relative to each element's node 0, are compared with the oracle at the origin in the
    large-rigid-motion parity test."""
    def rot(axis, deg):
        k = np.asarray(axis, float)
        k /= np.linalg.norm(k)
        t = np.radians(deg)
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * K @ K

    s = mesh.scene_cube(3, 3, 4, seed=2)
    X = s.mesh.nodes
    noise = np.random.default_rng(8).normal(0, 1e-5, X.size)
    out = {}
    for off in (0.0, 0.01, 10.0):
        x = (X @ rot((1, 2, 3), 75).T + off).ravel() + noise
        o = O.OracleModel.from_scene(s, gravity=(0.0, 0.0, 0.0), cg_tolerance=1e-12)
        o.set_state(x, np.zeros_like(x))
        assert o.step(1e-3, 3) == 0
        out[off] = o.state()[0] - x
    base = np.linalg.norm(out[0.0])
    assert np.linalg.norm(out[0.01] - out[0.0]) / base < 1e-8
    assert 1e-8 < np.linalg.norm(out[10.0] - out[0.0]) / base < 1e-5
