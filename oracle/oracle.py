"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is an FP64 CPU restatement of OpenSurgSim's corotational-tetrahedron implicit-Euler
step (see corotfem_oracle.cpp for the per-function citations). Only tests, the smoke check and
the benchmark's CPU-baseline leg import this module; the product never does.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libcorotfem_oracle.so")
_lib = None

ORC_OK, ORC_INVALID_ARG, ORC_DEGENERATE, ORC_CG_MAXITER, ORC_NONFINITE = 0, 1, 2, 3, 4


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("rayleigh_mass", ctypes.c_double),
        ("rayleigh_stiffness", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("gravity_enabled", ctypes.c_int32),
        ("newton_max_iterations", ctypes.c_int32),
        ("newton_epsilon", ctypes.c_double),
        ("cg_tolerance", ctypes.c_double),
        ("cg_max_iterations", ctypes.c_int32),
        ("element_type", ctypes.c_int32),   # 0 corotational tetrahedron, 1 linear tetrahedron, 2 hexahedron
        ("mass_lumping", ctypes.c_int32),   # FemRepresentation::setMassLumping
    ]


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("cg_iterations", ctypes.c_int32),
        ("newton_iterations", ctypes.c_int32),
        ("cg_converged", ctypes.c_int32),
        ("active", ctypes.c_int32),
        ("cg_error", ctypes.c_double),
        ("t_element", ctypes.c_double),
        ("t_system", ctypes.c_double),
        ("t_solve", ctypes.c_double),
        ("singular_g", ctypes.c_int32),
        ("invalid_rotation", ctypes.c_int32),
        ("orientation_warnings", ctypes.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile (g++ only)."""
    src = os.path.join(_HERE, "corotfem_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P, D, I32, I64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32), ctypes.c_int64
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_int32, D, ctypes.c_int32, I32, D, D, D, ctypes.c_int32, I32,
                                 ctypes.POINTER(OrcParams), I32]
        L.orc_destroy.argtypes = [P]
        L.orc_nnz.restype = I64
        L.orc_nnz.argtypes = [P]
        L.orc_step.restype = ctypes.c_int32
        L.orc_step.argtypes = [P, ctypes.c_double, ctypes.c_int32, ctypes.POINTER(OrcStats)]
        L.orc_get_state.argtypes = [P, D, D]
        L.orc_set_state.argtypes = [P, D, D]
        L.orc_get_pattern.argtypes = [P, I32, I32]
        L.orc_get_scatter.argtypes = [P, I32]
        L.orc_get_system.argtypes = [P, D, D, D, D, D, D]
        L.orc_get_mass_per_node.argtypes = [P, D]
        L.orc_get_element.argtypes = [P, ctypes.c_int32, D, D, D, D]
        L.orc_last_step_times.argtypes = [P, D]
        L.orc_last_step_times.restype = None
        L.orc_tet_compute.restype = ctypes.c_int32
        L.orc_tet_compute.argtypes = [D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D, D, D, D, D,
                                      D, D, I32]
        L.orc_polar.argtypes = [D, D, D]
        L.orc_hex_compute.restype = ctypes.c_int32
        L.orc_hex_compute.argtypes = [D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D, D, D]
        L.orc_hex_shape.argtypes = [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double, D]
        L.orc_add_external_force.restype = ctypes.c_int32
        L.orc_add_external_force.argtypes = [P, ctypes.c_int32, D, D, D, D]
        L.orc_apply_compliance.restype = ctypes.c_int32
        L.orc_apply_compliance.argtypes = [ctypes.c_void_p, ctypes.c_int32, D, D, ctypes.c_int32, I32]
        L.orc_cg_solve.restype = ctypes.c_int32
        L.orc_cg_solve.argtypes = [ctypes.c_int32, I32, I32, D, D, D, ctypes.c_double, ctypes.c_int32, I32, D]
        L.orc_masspoint_step.argtypes = [ctypes.c_double, ctypes.c_double, D, D, D, D]
        L.orc_step_many.restype = ctypes.c_int32
        L.orc_step_many.argtypes = [ctypes.POINTER(P), ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                    ctypes.c_int32]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class OracleError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"oracle status {status} {msg}")
        self.status = status


class OracleModel:
    """An OpenSurgSim-style Fem3DRepresentation (corotational or linear tets, implicit Euler, CG) on
    the CPU. element_type 1 selects Fem3DElementTetrahedron; its linear implicit Euler
    (OdeSolverLinearEulerImplicit) takes the same steps, the system matrix being constant.
    element_type 2 selects Fem3DElementCube: ``mesh.tets`` then holds 8 node ids per element."""

    def __init__(self, mesh, rayleigh_mass=0.0, rayleigh_stiffness=0.0, gravity=(0.0, -9.81, 0.0),
                 gravity_enabled=True, newton_max_iterations=1, newton_epsilon=1e-5, cg_tolerance=1e-10,
                 cg_max_iterations=0, element_type=0, mass_lumping=False):
        L = lib()
        self._nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float64).ravel()
        self._tets = np.ascontiguousarray(mesh.tets, dtype=np.int32).ravel()
        self._E = np.ascontiguousarray(mesh.young, dtype=np.float64)
        self._nu = np.ascontiguousarray(mesh.poisson, dtype=np.float64)
        self._rho = np.ascontiguousarray(mesh.density, dtype=np.float64)
        self._bc = np.ascontiguousarray(mesh.bc_dofs, dtype=np.int32)
        p = OrcParams()
        p.rayleigh_mass = rayleigh_mass
        p.rayleigh_stiffness = rayleigh_stiffness
        p.gravity[0], p.gravity[1], p.gravity[2] = gravity
        p.gravity_enabled = 1 if gravity_enabled else 0
        p.newton_max_iterations = newton_max_iterations
        p.newton_epsilon = newton_epsilon
        p.cg_tolerance = cg_tolerance
        p.cg_max_iterations = cg_max_iterations
        p.element_type = element_type
        p.mass_lumping = 1 if mass_lumping else 0
        st = ctypes.c_int32(0)
        self.num_nodes = mesh.nodes.shape[0]
        self.num_tets = mesh.tets.shape[0]
        self._npe = 8 if element_type == 2 else 4
        self.n = 3 * self.num_nodes
        self._h = L.orc_create(self.num_nodes, _d(self._nodes), self.num_tets, _i(self._tets), _d(self._E),
                               _d(self._nu), _d(self._rho), self._bc.size, _i(self._bc), ctypes.byref(p),
                               ctypes.byref(st))
        if not self._h:
            raise OracleError(st.value, "create failed")
        self.nnz = int(L.orc_nnz(self._h))
        self.last_stats = OrcStats()

    @classmethod
    def from_scene(cls, scene, **over):
        kw = dict(rayleigh_mass=scene.rayleigh_mass, rayleigh_stiffness=scene.rayleigh_stiffness,
                  gravity=scene.gravity, cg_tolerance=scene.cg_tolerance,
                  cg_max_iterations=scene.cg_max_iterations, element_type=scene.element_type)
        kw.update(over)
        return cls(scene.mesh, **kw)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def step(self, dt, nsteps=1):
        st = lib().orc_step(self._h, dt, nsteps, ctypes.byref(self.last_stats))
        return st

    def last_step_times(self):
        """Seconds of the last step: (element + assembly, system + BC + rhs, CG)."""
        t = np.zeros(3)
        lib().orc_last_step_times(self._h, _d(t))
        return t

    def state(self):
        x = np.empty(self.n)
        v = np.empty(self.n)
        lib().orc_get_state(self._h, _d(x), _d(v))
        return x, v

    def set_state(self, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        va = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_set_state(self._h, _d(xa) if xa is not None else None, _d(va) if va is not None else None)

    def pattern(self):
        colptr = np.empty(self.n + 1, dtype=np.int32)
        rowidx = np.empty(self.nnz, dtype=np.int32)
        lib().orc_get_pattern(self._h, _i(colptr), _i(rowidx))
        return colptr, rowidx

    def scatter(self):
        m = np.empty(self.num_tets * (3 * self._npe) ** 2, dtype=np.int32)
        lib().orc_get_scatter(self._h, _i(m))
        return m

    def system(self):
        """Last assembled S (BC applied), rhs, f, M, D, K in CSC order."""
        out = [np.empty(self.nnz), np.empty(self.n), np.empty(self.n), np.empty(self.nnz), np.empty(self.nnz),
               np.empty(self.nnz)]
        lib().orc_get_system(self._h, *[_d(a) for a in out])
        return dict(zip(["S", "rhs", "f", "M", "D", "K"], out))

    def add_external_force(self, element, coord, force, stiffness=None, damping=None):
        """Fem3DRepresentation::addExternalGeneralizedForce at element `element` (natural coordinates
        `coord`) for the next step: force (3), optional 3x3 stiffness and damping."""
        c = np.ascontiguousarray(coord, dtype=np.float64)
        F = np.ascontiguousarray(force, dtype=np.float64)
        K = np.ascontiguousarray(stiffness, dtype=np.float64).ravel() if stiffness is not None else None
        Dm = np.ascontiguousarray(damping, dtype=np.float64).ravel() if damping is not None else None
        st = lib().orc_add_external_force(self._h, int(element), _d(c), _d(F), _d(K) if K is not None else None,
                                          _d(Dm) if Dm is not None else None)
        if st != 0:
            raise OracleError(st, "add_external_force")

    def apply_compliance(self, B, warping=False):
        """DeformableRepresentation::applyCompliance on the columns of B (n x k) with the last step's
        system; with warping, FemRepresentation's compliance warping. Returns (X, status, iterations)."""
        B = np.asfortranarray(np.asarray(B, dtype=np.float64).reshape(self.n, -1))
        X = np.zeros_like(B, order="F")
        it = ctypes.c_int32(0)
        st = lib().orc_apply_compliance(self._h, B.shape[1], B.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        X.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1 if warping else 0,
                                        ctypes.byref(it))
        return X, st, it.value

    def mass_per_node(self):
        m = np.empty(self.num_nodes)
        lib().orc_get_mass_per_node(self._h, _d(m))
        return m

    def element(self, e):
        R, K, M, f = np.empty(9), np.empty(144), np.empty(144), np.empty(12)
        lib().orc_get_element(self._h, e, _d(R), _d(K), _d(M), _d(f))
        return R.reshape(3, 3), K.reshape(12, 12), M.reshape(12, 12), f


def tet_compute(x0, x, E, nu, rho):
    """Single-element rest precompute + corotational update; returns a dict of arrays."""
    x0 = np.ascontiguousarray(x0, dtype=np.float64).ravel()
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = {k: np.empty(s) for k, s in [("Vinv", 16), ("K0", 144), ("M0", 144), ("vol", 1), ("R", 9), ("K", 144),
                                       ("M", 144), ("f", 12)]}
    ow = ctypes.c_int32(0)
    st = lib().orc_tet_compute(_d(x0), _d(x), E, nu, rho, _d(out["Vinv"]), _d(out["K0"]), _d(out["M0"]),
                               _d(out["vol"]), _d(out["R"]), _d(out["K"]), _d(out["M"]), _d(out["f"]),
                               ctypes.byref(ow))
    if st != ORC_OK:
        raise OracleError(st, "tet_compute")
    res = dict(Vinv=out["Vinv"].reshape(4, 4), K0=out["K0"].reshape(12, 12), M0=out["M0"].reshape(12, 12),
               vol=float(out["vol"][0]), R=out["R"].reshape(3, 3), K=out["K"].reshape(12, 12),
               M=out["M"].reshape(12, 12), f=out["f"], orientation_warning=bool(ow.value))
    return res


def hex_compute(x0, x, E, nu, rho):
    """One Fem3DElementCube: rest volume, K (24x24), M (24x24) and f = -K (x - x0). Raises
    OracleError(2) where the reference's initialize asserts (singular Jacobian, volume <= 1e-12)."""
    x0 = np.ascontiguousarray(x0, dtype=np.float64).ravel()
    x = np.ascontiguousarray(x if x is not None else x0, dtype=np.float64).ravel()
    vol = np.zeros(1)
    K = np.zeros((24, 24))
    M = np.zeros((24, 24))
    f = np.zeros(24)
    st = lib().orc_hex_compute(_d(x0), _d(x), E, nu, rho, _d(vol), _d(K), _d(M), _d(f))
    if st != 0:
        raise OracleError(st, "hexahedron initialize failed")
    return dict(volume=float(vol[0]), K=K, M=M, f=f)


def hex_shape(i, eps, eta, mu):
    """(N_i, dN_i/deps, dN_i/deta, dN_i/dmu) of Fem3DElementCube at a natural coordinate."""
    out = np.zeros(4)
    lib().orc_hex_shape(i, eps, eta, mu, _d(out))
    return out


def polar(F):
    F = np.ascontiguousarray(F, dtype=np.float64).ravel()
    R, S = np.empty(9), np.empty(9)
    lib().orc_polar(_d(F), _d(R), _d(S))
    return R.reshape(3, 3), S.reshape(3, 3)


def cg_solve(colptr, rowidx, vals, b, tol=np.finfo(float).eps, max_iter=0):
    colptr = np.ascontiguousarray(colptr, dtype=np.int32)
    rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    it = ctypes.c_int32(0)
    err = ctypes.c_double(0)
    st = lib().orc_cg_solve(b.size, _i(colptr), _i(rowidx), _d(vals), _d(b), _d(x), tol, max_iter,
                            ctypes.byref(it), ctypes.byref(err))
    return x, it.value, err.value, st


def masspoint_step(viscosity, dt, x0, v0):
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    x1, v1 = np.empty(3), np.empty(3)
    lib().orc_masspoint_step(viscosity, dt, _d(x0), _d(v0), _d(x1), _d(v1))
    return x1, v1


def step_many(models, dt, nsteps, threads):
    arr = (ctypes.c_void_p * len(models))(*[m.handle for m in models])
    return lib().orc_step_many(arr, len(models), dt, nsteps, threads)
