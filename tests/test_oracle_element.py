"""The oracle's element math against the reference's own known-answer tests (CPU).

Restated from SurgSim/Physics/UnitTests/Fem3DElementTetrahedronTests.cpp and
Fem3DElementCorotationalTetrahedronTests.cpp; the host build of the GPU element math
(tests/support/element_host.cu) is checked against the same cases.
"""

import numpy as np
import pytest

from oracle import oracle as O


def approx(a, b, prec=1e-12):
    """Eigen's isApprox: |a - b| <= prec * min(|a|, |b|)."""
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))


def rot(angle, axis):
    axis = np.asarray(axis, float)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def blockdiag4(R):
    out = np.zeros((12, 12))
    for a in range(4):
        out[3 * a:3 * a + 3, 3 * a:3 * a + 3] = R
    return out


# Fem3DElementTetrahedronTests.cpp:110-247: tet of a unit cube at (0.1, 1.2, 2.3), rho 1000, E 1e6, nu 0.45.
TET_X0 = np.array([[0.1, 1.2, 2.3], [1.1, 1.2, 2.3], [0.1, 2.2, 2.3], [0.1, 1.2, 3.3]])
RHO, E, NU = 1000.0, 1e6, 0.45


def expected_mass(vol):
    M = 2.0 * np.eye(12)
    for d in (3, 6, 9):
        M += np.eye(12, k=d) + np.eye(12, k=-d)
    return M * RHO * vol / 20.0


def expected_stiffness_B(vol):
    # hand-derived B (bi = {-1 1 0 0}, ci = {-1 0 1 0}, di = {-1 0 0 1}) and E (:159-196)
    B = np.zeros((6, 12))
    for (r, c, v) in [(0, 0, -1), (0, 3, 1), (1, 1, -1), (1, 7, 1), (2, 2, -1), (2, 11, 1), (3, 0, -1), (3, 1, -1),
                      (3, 4, 1), (3, 6, 1), (4, 1, -1), (4, 2, -1), (4, 8, 1), (4, 10, 1), (5, 0, -1), (5, 2, -1),
                      (5, 5, 1), (5, 9, 1)]:
        B[r, c] = v
    B *= 1.0 / (6.0 * vol)
    Em = np.zeros((6, 6))
    Em[:3, :3] = NU
    np.fill_diagonal(Em[:3, :3], 1.0 - NU)
    Em[3:, 3:] = np.diag([0.5 - NU] * 3)
    Em *= E / ((1.0 + NU) * (1.0 - 2.0 * NU))
    return vol * B.T @ Em @ B


def expected_stiffness_afem():
    # closed form of the AFEM Ch.9 notes (:199-247)
    e = E / (12.0 * (1.0 - 2.0 * NU) * (1.0 + NU))
    n0, n1 = 1.0 - 2.0 * NU, 1.0 - NU
    K = np.zeros((12, 12))
    K[0, 1] = K[0, 2] = K[1, 2] = 1.0
    vals = {(0, 3): -2 * n1, (0, 4): -n0, (0, 5): -n0, (1, 3): -2 * NU, (1, 4): -n0, (2, 3): -2 * NU, (2, 5): -n0,
            (0, 6): -n0, (0, 7): -2 * NU, (1, 6): -n0, (1, 7): -2 * n1, (1, 8): -n0, (2, 7): -2 * NU, (2, 8): -n0,
            (0, 9): -n0, (0, 11): -2 * NU, (1, 10): -n0, (1, 11): -2 * NU, (2, 9): -n0, (2, 10): -n0,
            (2, 11): -2 * n1, (3, 7): 2 * NU, (3, 11): 2 * NU, (4, 6): n0, (5, 9): n0, (7, 11): 2 * NU,
            (8, 10): n0}
    for (r, c), v in vals.items():
        K[r, c] = v
    K = K + K.T
    for i in range(3):
        K[i, i] = 4.0 - 6.0 * NU
    for i in range(3, 12):
        K[i, i] = n0
    K[3, 3] = K[7, 7] = K[11, 11] = 2.0 * n1
    return K * e


def test_tet_volume_mass_stiffness_known_answers():
    r = O.tet_compute(TET_X0, TET_X0, E, NU, RHO)
    assert abs(r["vol"] - 1.0 / 6.0) < 1e-10  # Fem3DElementTetrahedronTests.cpp:275-282
    assert approx(r["M0"], expected_mass(1.0 / 6.0))
    assert approx(r["K0"], expected_stiffness_B(1.0 / 6.0))
    assert approx(r["K0"], expected_stiffness_afem())
    assert not r["orientation_warning"]


def test_tet_orientation_warning_and_degenerate():
    swapped = TET_X0[[0, 2, 1, 3]]
    r = O.tet_compute(swapped, swapped, E, NU, RHO)
    assert r["orientation_warning"]
    assert r["vol"] < 0  # the reference keeps the signed volume (Fem3DElementTetrahedron.cpp:230-234)
    flat = TET_X0.copy()
    flat[3] = flat[2]
    with pytest.raises(O.OracleError) as e:
        O.tet_compute(flat, flat, E, NU, RHO)
    assert e.value.status == O.ORC_DEGENERATE  # Fem3DElementCorotationalTetrahedron.cpp:66-72


# Fem3DElementCorotationalTetrahedronTests.cpp:106-159
COROT_X0 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
ROT = rot(4.1415, [1.0, 0.2, -0.3])
TRANS = np.array([1.2, 2.3, 3.4])
DELTA = np.array([[0.01, -0.02, 0.005], [-0.01, -0.01, -0.03], [0.0, -0.015, 0.03]])


def transformed(linear, translation, deform=False):
    x = (linear @ COROT_X0.T).T + translation
    if deform:
        x = x + DELTA[np.arange(4) % 3]
    return x


@pytest.mark.parametrize("case", ["identity", "translation", "rotation", "rotation+translation", "rotation*scale"])
def test_corotational_rotation_mass_stiffness(case):
    """ComputeRotationMassAndStiffnessTest (:232-336)."""
    lin, tr = {"identity": (np.eye(3), 0 * TRANS), "translation": (np.eye(3), TRANS),
               "rotation": (ROT, 0 * TRANS), "rotation+translation": (ROT, TRANS),
               "rotation*scale": (ROT * 45.3, TRANS)}[case]
    r = O.tet_compute(COROT_X0, transformed(lin, tr), E, NU, RHO)
    R12 = blockdiag4(r["R"])
    if case in ("identity", "translation"):
        assert approx(r["R"], np.eye(3))
        assert approx(r["K"], r["K0"])
        assert approx(r["M"], r["M0"])
    else:
        assert approx(r["R"], ROT)
        assert approx(r["M"], R12 @ r["M0"] @ R12.T)
        assert not approx(r["K"], r["K0"])
        if case == "rotation*scale":
            assert not approx(r["K"], R12 @ r["K0"] @ R12.T)
        else:
            assert approx(r["K"], R12 @ r["K0"] @ R12.T)


@pytest.mark.parametrize("rigid", [False, True])
@pytest.mark.parametrize("deform", [False, True])
def test_corotational_force(rigid, deform):
    """AddForceTest (:524-611): f = -R K0 R^T (x - R x0) within 1e-8."""
    lin, tr = (ROT, TRANS) if rigid else (np.eye(3), 0 * TRANS)
    x = transformed(lin, tr, deform)
    r = O.tet_compute(COROT_X0, x, E, NU, RHO)
    R12 = blockdiag4(r["R"])
    expected = -R12 @ r["K0"] @ R12.T @ (x.ravel() - R12 @ COROT_X0.ravel())
    assert np.linalg.norm(r["f"] - expected) < 1e-8
    if not deform:
        assert np.abs(r["f"]).max() < 1e-8


def test_add_matvec():
    """AddMatVecTest (:613-683): 1.4 M 1 + 1.6 K 1 through the element matrices."""
    x = transformed(ROT, TRANS, True)
    r = O.tet_compute(COROT_X0, x, E, NU, RHO)
    ones = np.ones(12)
    expected = (1.4 * r["M"] + 1.6 * r["K"]) @ ones
    got = 1.4 * (r["M"] @ ones) + 1.6 * (r["K"] @ ones)
    assert np.linalg.norm(got - expected) <= 1e-10 * np.linalg.norm(expected)


def test_polar_proper_rotation_for_reflections():
    """det F < 0: proper rotation with the reflection on the smallest singular value."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        U = rot(rng.uniform(0, 3), rng.standard_normal(3))
        V = rot(rng.uniform(0, 3), rng.standard_normal(3))
        s = np.sort(rng.uniform(0.5, 2.0, 3))[::-1]
        F = U @ np.diag([s[0], s[1], -s[2]]) @ V.T
        R, S = O.polar(F)
        assert abs(np.linalg.det(R) - 1.0) < 1e-12
        assert np.allclose(R @ S, F, atol=1e-12)
        assert np.allclose(S, S.T, atol=1e-12)
        assert np.allclose(R, U @ V.T, atol=1e-10)
