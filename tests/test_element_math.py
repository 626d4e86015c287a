"""The GPU element math (gbfem_element.cuh), compiled for the host, against the oracle (CPU)."""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "support", "element_host.cu")
LIB = os.path.join(HERE, "support", "libelemhost.so")


@pytest.fixture(scope="module")
def elem():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    deps = [SRC] + [os.path.join(ROOT, "opensurgsim_gb300", "csrc", f)
                    for f in ("gbfem_element.cuh", "gbfem_adjoint.cuh", "gbfem_dual.cuh")]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(d) for d in deps):
        subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                        "-I" + os.path.join(ROOT, "opensurgsim_gb300", "csrc"), "-o", LIB, SRC], check=True,
                       capture_output=True)
    L = ctypes.CDLL(LIB)
    D = ctypes.POINTER(ctypes.c_double)
    L.gbfem_host_element.argtypes = [ctypes.c_int, D, D, D, D, D, ctypes.POINTER(ctypes.c_int)] + \
        [ctypes.c_double] * 6 + [D, D, D, D]
    L.gbfem_host_element.restype = ctypes.c_int
    L.gbfem_host_adjoint_element.argtypes = [D, D, D, ctypes.POINTER(ctypes.c_int)] + [ctypes.c_double] * 6 + \
        [D] * 7
    L.gbfem_host_adjoint_element.restype = ctypes.c_int
    L.gbfem_host_poisson_partials.argtypes = [ctypes.c_double, ctypes.c_double, D, D]
    L.gbfem_host_poisson_partials.restype = None

    def run(fp32, x0, x, v=None, E=1e6, nu=0.45, rho=1000.0, dt=1e-3, alpha=0.0, beta=0.0, nd=(0, 1, 2, 3)):
        def d(a):
            return np.ascontiguousarray(a, dtype=np.float64).ravel()
        x0, x = d(x0), d(x)
        v = np.zeros(12) if v is None else d(v)
        K, rhs, f, R = np.zeros(144), np.zeros(12), np.zeros(12), np.zeros(9)
        p = lambda a: a.ctypes.data_as(D)  # noqa: E731
        fl = L.gbfem_host_element(fp32, p(x0), p(x), p(v), p(x), p(v), (ctypes.c_int * 4)(*nd), E, nu, rho, dt,
                                  alpha, beta, p(K), p(rhs), p(f), p(R))
        assert fl >= 0
        return K.reshape(12, 12), f, rhs, R.reshape(3, 3), fl

    def adjoint(x0, x, v, mu, dv, E=1e5, nu=0.45, rho=1000.0, dt=1e-3, alpha=0.01, beta=0.001, nd=(0, 1, 2, 3)):
        def d(a):
            return np.ascontiguousarray(a, dtype=np.float64).ravel()
        x0, x, v, mu, dv = d(x0), d(x), d(v), d(mu), d(dv)
        psi, pl, pm = (ctypes.c_double() for _ in range(3))
        gx, gv = np.zeros(12), np.zeros(12)
        p = lambda a: a.ctypes.data_as(D)  # noqa: E731
        r = L.gbfem_host_adjoint_element(p(x0), p(x), p(v), (ctypes.c_int * 4)(*nd), E, nu, rho, dt, alpha, beta,
                                         p(mu), p(dv), ctypes.byref(psi), p(gx), p(gv), ctypes.byref(pl),
                                         ctypes.byref(pm))
        assert r == 0
        return psi.value, gx, gv, pl.value, pm.value

    def poisson_partials(lamV, muV):
        dl, dm = ctypes.c_double(), ctypes.c_double()
        L.gbfem_host_poisson_partials(lamV, muV, ctypes.byref(dl), ctypes.byref(dm))
        return dl.value, dm.value

    run.adjoint = adjoint
    run.poisson_partials = poisson_partials
    return run


def rot(angle, axis):
    axis = np.asarray(axis, float)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


X0 = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
ROT = rot(4.1415, [1.0, 0.2, -0.3])
DELTA = np.array([[0.01, -0.02, 0.005], [-0.01, -0.01, -0.03], [0.0, -0.015, 0.03]])


@pytest.mark.parametrize("case", ["identity", "rotation+translation", "deformed", "scale45"])
def test_fp64_element_matches_oracle(elem, case):
    x = {"identity": X0, "rotation+translation": (ROT @ X0.T).T + [1.2, 2.3, 3.4],
         "deformed": (ROT @ X0.T).T + [1.2, 2.3, 3.4] + DELTA[np.arange(4) % 3],
         "scale45": (45.3 * ROT @ X0.T).T + [1.2, 2.3, 3.4]}[case]
    o = O.tet_compute(X0, x, 1e6, 0.45, 1000.0)
    K, f, rhs, R, fl = elem(0, X0, x)
    assert fl == 0
    assert np.abs(K - o["K"]).max() <= 1e-13 * np.abs(o["K"]).max()  # includes the KTimesRx_x0 quirk
    assert np.abs(R - o["R"]).max() < 1e-13
    # the reference's force test uses an absolute 1e-8 (epsilonAddForce); rigid motions leave only
    # rounding noise, which is smaller here (relative coordinates) than in the oracle
    assert np.linalg.norm(f - o["f"]) <= max(1e-8, 1e-12 * np.linalg.norm(o["f"]))


def test_tangent_is_not_symmetric_like_the_reference(elem):
    x = (ROT @ X0.T).T + DELTA[np.arange(4) % 3] * 3
    K, *_ = elem(0, X0, x)
    o = O.tet_compute(X0, x, 1e6, 0.45, 1000.0)
    asym = np.abs(o["K"] - o["K"].T).max() / np.abs(o["K"]).max()
    assert asym > 1e-6  # the reference's tangent is non-symmetric (rotated stiffness in KTimesRx_x0)
    assert np.abs((K - K.T) - (o["K"] - o["K"].T)).max() <= 1e-12 * np.abs(o["K"]).max()


def test_rhs_combines_force_damping_and_implicit_terms(elem):
    """rhs_e = f_e + K_e (-(beta + dt) v) + M0 (-alpha v) on the first Newton iteration."""
    rng = np.random.default_rng(7)
    x = X0 * 0.01 + rng.normal(0, 2e-4, (4, 3))
    v = rng.normal(0, 0.05, 12)
    dt, a, b = 1e-3, 0.01, 0.001
    o = O.tet_compute(X0 * 0.01, x, 1e5, 0.45, 1000.0)
    K, f, rhs, R, fl = elem(0, X0 * 0.01, x, v, E=1e5, dt=dt, alpha=a, beta=b)
    expected = o["f"] + o["K"] @ (-(b + dt) * v) + o["M"] @ (-a * v)
    assert np.linalg.norm(rhs - expected) <= 1e-10 * np.linalg.norm(expected)


def test_fp32_element_accuracy(elem):
    """Mixed form: FP32 tangent to ~1e-7 and FP32 force to ~1e-7 relative on realistic elements
    (h = 4 mm, 1% strain, rotated), thanks to the FP64 Gram-difference strain."""
    rng = np.random.default_rng(1)
    ek, ef = [], []
    for _ in range(100):
        h = 0.004
        xr = X0 * h + rng.uniform(-0.1 * h, 0.1 * h, (4, 3)) + rng.uniform(0, 0.1, 3)
        F = np.eye(3) + 1e-2 * rng.standard_normal((3, 3))
        Rm = rot(rng.uniform(0, 0.3), rng.standard_normal(3))
        c = xr.mean(0)
        x = ((Rm @ F) @ (xr - c).T).T + c
        o = O.tet_compute(xr, x, 1e5, 0.45, 1000.0)
        K, f, rhs, R, fl = elem(1, xr, x, E=1e5)
        ek.append(np.abs(K - o["K"]).max() / np.abs(o["K"]).max())
        ef.append(np.linalg.norm(f - o["f"]) / np.linalg.norm(o["f"]))
    print("fp32 K rel err median %.2e max %.2e; f median %.2e max %.2e" % (np.median(ek), max(ek), np.median(ef),
                                                                           max(ef)))
    assert np.median(ek) < 5e-7 and max(ek) < 2e-6
    assert np.median(ef) < 5e-7 and max(ef) < 1e-5


def test_inverted_element_takes_svd_fallback(elem):
    x = X0.copy()
    x[3, 2] = -0.5  # node 3 pushed through the opposite face: det F < 0
    K, f, rhs, R, fl = elem(0, X0, x)
    assert fl & 1
    o = O.tet_compute(X0, x, 1e6, 0.45, 1000.0)
    assert abs(np.linalg.det(R) - 1) < 1e-12
    assert np.abs(R - o["R"]).max() < 1e-10
    assert np.abs(K - o["K"]).max() <= 1e-10 * np.abs(o["K"]).max()


@pytest.mark.parametrize("fp32", [0, 1])
def test_collapsed_element_takes_the_singular_g_early_return(elem, fp32):
    """All four nodes on one line: F has rank 1, G = (tr(S) I - S) R^T is singular, and the reference
    returns from computeRotationMassAndStiffness after forming K = R K0 R^T, without the dR/dx terms
    (Fem3DElementCorotationalTetrahedron.cpp:199-216); the force is then -K (x - R x0) = -R K0 w with
    w = R^T p - q (:103-113). The rotation of a rank-1 F is not unique (any completion of its
    singular vectors is a polar factor), so the check holds for the R the element code returns. The
    FP32 form routes such an element to its FP64 SVD path, where G is decided in FP64."""
    h = 0.01
    x0 = X0 * h
    d = np.array([0.3, 0.5, 0.8]) / np.linalg.norm([0.3, 0.5, 0.8])
    x = np.stack([t * d for t in (0.0, 0.004, 0.007, 0.011)]) + 0.02
    E, nu = 1e5, 0.45
    K, f, rhs, R, fl = elem(fp32, x0, x, E=E, nu=nu)
    assert fl & 2 and fl & 1  # singular G, on the SVD path
    assert abs(np.linalg.det(R) - 1) < (1e-6 if fp32 else 1e-12)
    Vh = np.c_[x0, np.ones(4)].T
    g = np.linalg.inv(Vh)[:, :3]  # shape-function gradients, one row per node
    vol = abs(np.linalg.det(x0[1:] - x0[0])) / 6
    lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    K0 = np.zeros((12, 12))
    for a in range(4):
        for b in range(4):
            K0[3 * a:3 * a + 3, 3 * b:3 * b + 3] = vol * (lam * np.outer(g[a], g[b]) + mu * np.outer(g[b], g[a]) +
                                                          mu * (g[a] @ g[b]) * np.eye(3))
    R12 = np.kron(np.eye(4), R)
    Krot = R12 @ K0 @ R12.T
    tol = 2e-6 if fp32 else 1e-12
    assert np.abs(K - Krot).max() <= tol * np.abs(Krot).max()
    w = ((x - x[0]) @ R) - (x0 - x0[0])  # R^T p_a - q_a per node (rows)
    fe = -(R12 @ K0 @ w.ravel())
    assert np.linalg.norm(f - fe) <= (1e-5 if fp32 else 1e-12) * np.linalg.norm(fe)


def _adjoint_case(seed):
    rng = np.random.default_rng(seed)
    x0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float) * 0.01 + rng.uniform(-1e-3, 1e-3, (4, 3))
    R = rot(0.7, [1.0, 2.0, 0.5])
    x = (x0 @ R.T) * 1.05 + rng.uniform(-5e-4, 5e-4, (4, 3)) + 0.02
    v = rng.normal(0, 0.05, (4, 3))
    mu = rng.normal(0, 1.0, 12)
    dv = rng.normal(0, 0.01, 12)
    nd = tuple(int(i) for i in rng.permutation([3, 7, 11, 19]))
    return x0, x, v, mu, dv, nd


def _inverted_case(seed):
    """An element turned inside out (F = R diag(1.1, 0.9, -0.8) plus noise, det F < 0): its rotation
    comes from the SVD path, and S = R^T F is indefinite."""
    x0, _, v, mu, dv, nd = _adjoint_case(seed)
    R = rot(0.4, [0.3, -1.0, 2.0])
    rng = np.random.default_rng(seed + 100)
    F = R @ np.diag([1.1, 0.9, -0.8])
    x = x0[0] + (x0 - x0[0]) @ F.T + rng.uniform(-2e-4, 2e-4, (4, 3)) + 0.01
    assert np.linalg.det((x[1:] - x[0]).T) < 0
    return x0, x, v, mu, dv, nd


@pytest.mark.parametrize("seed,inverted", [(0, False), (1, False), (2, False), (0, True), (4, True)])
def test_element_adjoint_position_gradient_matches_central_differences(elem, seed, inverted):
    """d psi_e / d x_e from the dual-number passes (the rotation's derivative from the polar
    factor's tangent) vs central differences of psi_e (the element share of mu.rhs - mu.S dv that
    the step's adjoint differentiates), on regular and inverted elements."""
    x0, x, v, mu, dv, nd = (_inverted_case if inverted else _adjoint_case)(seed)
    _, gx, _, _, _ = elem.adjoint(x0, x, v, mu, dv, nd=nd)
    h = 1e-7
    fd = np.zeros(12)
    for j in range(12):
        xp, xm = x.copy().ravel(), x.copy().ravel()
        xp[j] += h
        xm[j] -= h
        fd[j] = (elem.adjoint(x0, xp, v, mu, dv, nd=nd)[0] - elem.adjoint(x0, xm, v, mu, dv, nd=nd)[0]) / (2 * h)
    assert np.linalg.norm(gx - fd) <= 1e-6 * np.linalg.norm(fd)


@pytest.mark.parametrize("seed", [0, 3])
def test_element_adjoint_velocity_and_modulus_gradients(elem, seed):
    x0, x, v, mu, dv, nd = _adjoint_case(seed)
    E, nu = 2.5e5, 0.42
    psi, _, gv, pl, pm = elem.adjoint(x0, x, v, mu, dv, E=E, nu=nu, nd=nd)
    h = 1e-6
    fd = np.zeros(12)
    for j in range(12):
        vp, vm = v.copy().ravel(), v.copy().ravel()
        vp[j] += h
        vm[j] -= h
        fd[j] = (elem.adjoint(x0, x, vp, mu, dv, E=E, nu=nu, nd=nd)[0] -
                 elem.adjoint(x0, x, vm, mu, dv, E=E, nu=nu, nd=nd)[0]) / (2 * h)
    assert np.linalg.norm(gv - fd) <= 1e-8 * np.linalg.norm(fd)
    # log E: psi's elastic part is homogeneous of degree one in (lambda V, mu V).
    vol = abs(np.linalg.det(np.c_[x0[1:] - x0[0]])) / 6
    lamV = E * nu / ((1 + nu) * (1 - 2 * nu)) * vol
    muV = E / (2 * (1 + nu)) * vol
    hE = 1e-6
    fdE = (elem.adjoint(x0, x, v, mu, dv, E=E * np.exp(hE), nu=nu, nd=nd)[0] -
           elem.adjoint(x0, x, v, mu, dv, E=E * np.exp(-hE), nu=nu, nd=nd)[0]) / (2 * hE)
    assert abs(lamV * pl + muV * pm - fdE) <= 1e-7 * abs(fdE)


@pytest.mark.parametrize("seed,nu", [(0, 0.45), (1, 0.30), (3, 0.49)])
def test_element_adjoint_poisson_gradient_matches_central_differences(elem, seed, nu):
    """d psi_e / d nu at fixed E: the element's partials in (lambda V, mu V) times the kernel's chain
    rule (adj::poisson_partials, the code k_element_adjoint runs) against central differences of
    psi_e in nu (nu enters K0 through lambda and mu, Fem3DElementTetrahedron.cpp:204-205)."""
    x0, x, v, mu, dv, nd = _adjoint_case(seed)
    E = 2.5e5
    _, _, _, pl, pm = elem.adjoint(x0, x, v, mu, dv, E=E, nu=nu, nd=nd)
    vol = abs(np.linalg.det(np.c_[x0[1:] - x0[0]])) / 6
    lamV = E * nu / ((1 + nu) * (1 - 2 * nu)) * vol
    muV = E / (2 * (1 + nu)) * vol
    dl, dm = elem.poisson_partials(lamV, muV)
    g = dl * pl + dm * pm
    h = 1e-6
    fd = (elem.adjoint(x0, x, v, mu, dv, E=E, nu=nu + h, nd=nd)[0] -
          elem.adjoint(x0, x, v, mu, dv, E=E, nu=nu - h, nd=nd)[0]) / (2 * h)
    assert abs(g - fd) <= 1e-6 * abs(fd), (g, fd)
