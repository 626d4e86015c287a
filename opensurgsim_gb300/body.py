"""One deformable body on the GPU: a thin Python handle over the gbfem C ABI."""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GbfemError, dptr, iptr


class Body:
    """A corotational-tetrahedron body stepped by backward Euler + Jacobi-PCG on one GPU.

    Mirrors ``FemRepresentation::update`` semantics (``FemRepresentation.cpp:232-294``): one
    Newton iteration by default, CG reading the lower triangle, boundary-condition dofs fixed, the
    body deactivated when its state stops being finite.
    """

    def __init__(self, mesh, rayleigh_mass=0.0, rayleigh_stiffness=0.0, gravity=(0.0, -9.81, 0.0),
                 gravity_enabled=True, newton_max_iterations=1, newton_epsilon=1e-5,
                 cg_tolerance=np.finfo(float).eps, cg_max_iterations=0, precision=_lib.PRECISION_FP64, device=0,
                 autotune=False, element_type=_lib.ELEMENT_COROTATIONAL_TET, mass_lumping=False):
        """`mesh` is one TetMesh, or a list of them for a batch (mixed precision only). With
        element_type ELEMENT_HEXAHEDRON, ``mesh.tets`` holds 8 node ids per element. mass_lumping is
        FemRepresentation::setMassLumping (every row of M summed onto its diagonal)."""
        L = _lib.load()
        self.nodes_per_element = 8 if element_type == _lib.ELEMENT_HEXAHEDRON else 4
        meshes = list(mesh) if isinstance(mesh, (list, tuple)) else [mesh]
        self._keep = []
        descs = (_lib.MeshDesc * len(meshes))()
        for k, m in enumerate(meshes):
            arrs = [np.ascontiguousarray(m.nodes, dtype=np.float64).ravel(),
                    np.ascontiguousarray(m.tets, dtype=np.int32).ravel(),
                    np.ascontiguousarray(m.young, dtype=np.float64), np.ascontiguousarray(m.poisson, dtype=np.float64),
                    np.ascontiguousarray(m.density, dtype=np.float64),
                    np.ascontiguousarray(m.bc_dofs, dtype=np.int32)]
            self._keep.append(arrs)
            d = descs[k]
            d.num_nodes = arrs[0].size // 3
            d.rest_positions = dptr(arrs[0])
            d.num_tets = arrs[1].size // self.nodes_per_element
            d.tets = iptr(arrs[1])
            d.young_modulus = dptr(arrs[2])
            d.poisson_ratio = dptr(arrs[3])
            d.mass_density = dptr(arrs[4])
            d.num_bc_dofs = arrs[5].size
            d.bc_dofs = iptr(arrs[5]) if arrs[5].size else None
        p = _lib.Params()
        L.gbfem_params_default(ctypes.byref(p))
        p.rayleigh_mass = rayleigh_mass
        p.rayleigh_stiffness = rayleigh_stiffness
        p.gravity[0], p.gravity[1], p.gravity[2] = gravity
        p.gravity_enabled = 1 if gravity_enabled else 0
        p.newton_max_iterations = newton_max_iterations
        p.newton_epsilon = newton_epsilon
        p.cg_tolerance = cg_tolerance
        p.cg_max_iterations = cg_max_iterations
        p.precision = precision
        p.device = device
        p.autotune = 1 if autotune else 0
        p.element_type = element_type
        p.mass_lumping = 1 if mass_lumping else 0
        self.params = p
        h = ctypes.c_void_p()
        if len(meshes) == 1 and not isinstance(mesh, (list, tuple)):
            st = L.gbfem_create(ctypes.byref(descs[0]), ctypes.byref(p), ctypes.byref(h))
        else:
            st = L.gbfem_batch_create(len(meshes), descs, ctypes.byref(p), ctypes.byref(h))
        if st != _lib.GBFEM_OK:
            raise GbfemError(st, _lib.last_error(None))
        self._h = h
        self.num_meshes = len(meshes)
        self.num_nodes = sum(d.num_nodes for d in descs)
        self.num_tets = sum(d.num_tets for d in descs)
        n, nnz = ctypes.c_int64(), ctypes.c_int64()
        L.gbfem_get_sizes(h, ctypes.byref(n), ctypes.byref(nnz))
        self.n = n.value
        self.nnz = nnz.value
        self.node_offsets = np.zeros(self.num_meshes + 1, dtype=np.int32)
        self.tet_offsets = np.zeros(self.num_meshes + 1, dtype=np.int32)
        self.nnz_per_mesh = np.zeros(self.num_meshes, dtype=np.int64)
        L.gbfem_batch_info(h, None, iptr(self.node_offsets), iptr(self.tet_offsets),
                           self.nnz_per_mesh.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        self.last_status = _lib.GBFEM_OK

    def segment_stats(self):
        """Per mesh over the last step call: iterations, refreshes, converged, worst relative residual."""
        k = self.num_meshes
        it, rf, cv = (np.zeros(k, dtype=np.int32) for _ in range(3))
        res = np.zeros(k)
        _lib.load().gbfem_batch_segment_stats(self._h, iptr(it), iptr(rf), iptr(cv), dptr(res))
        return dict(iterations=it, refreshes=rf, converged=cv, relative_residual=res)

    def add_external_force(self, element, coord, force, stiffness=None, damping=None):
        """Fem3DRepresentation::addExternalGeneralizedForce for the next step: a force (3) at the point
        of `element` with natural coordinates `coord`, optional 3x3 stiffness and damping."""
        c = np.ascontiguousarray(coord, dtype=np.float64)
        F = np.ascontiguousarray(force, dtype=np.float64)
        K = np.ascontiguousarray(stiffness, dtype=np.float64).ravel() if stiffness is not None else None
        Dm = np.ascontiguousarray(damping, dtype=np.float64).ravel() if damping is not None else None
        self._check(_lib.load().gbfem_add_external_force(self._h, int(element), dptr(c), dptr(F),
                                                         dptr(K) if K is not None else None,
                                                         dptr(Dm) if Dm is not None else None))

    def apply_compliance(self, B, warping=False):
        """Solve the last step's system for the columns of B (n x k): applyCompliance semantics (BC rows
        zeroed in and out), optionally with compliance warping. Returns (X, status, iterations)."""
        B = np.asfortranarray(np.asarray(B, dtype=np.float64).reshape(self.n, -1))
        X = np.zeros_like(B, order="F")
        it = ctypes.c_int32(0)
        st = _lib.load().gbfem_apply_compliance(self._h, B.shape[1], B.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                X.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                _lib.COMPLIANCE_WARPING if warping else 0, ctypes.byref(it))
        if st not in (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER):
            raise GbfemError(st, _lib.last_error(self._h))
        return X, st, it.value

    def tuning(self):
        """(elements per block, CTAs per SM, refresh weight, CG schedule) of the mixed form's kernels;
        the schedule is one of _lib.CG_TWO_PHASE, CG_ONE_PHASE, CG_FP64."""
        e, c, r, g = (ctypes.c_int32() for _ in range(4))
        self._check(_lib.load().gbfem_get_tuning(self._h, ctypes.byref(e), ctypes.byref(c), ctypes.byref(r),
                                                 ctypes.byref(g)))
        return e.value, c.value, r.value, g.value

    def set_tuning(self, elems_per_block, ctas_per_sm, refresh_weight, cg_schedule=-1):
        """Pins the tuning (and stops autotuning); cg_schedule -1 keeps the handle's schedule."""
        self._check(_lib.load().gbfem_set_tuning(self._h, int(elems_per_block), int(ctas_per_sm), int(refresh_weight),
                                                 int(cg_schedule)))

    @classmethod
    def from_scene(cls, scene, **over):
        kw = dict(rayleigh_mass=scene.rayleigh_mass, rayleigh_stiffness=scene.rayleigh_stiffness,
                  gravity=scene.gravity, cg_tolerance=scene.cg_tolerance, cg_max_iterations=scene.cg_max_iterations,
                  element_type=scene.element_type)
        kw.update(over)
        return cls(scene.mesh, **kw)

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().gbfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, st, allow=()):
        if st != _lib.GBFEM_OK and st not in allow:
            raise GbfemError(st, _lib.last_error(self._h))
        return st

    def step(self, dt, nsteps=1, flags=0, raise_on=(_lib.GBFEM_CUDA_ERROR, _lib.GBFEM_OUT_OF_MEMORY,
                                                   _lib.GBFEM_INVALID_ARG)):
        """Advance nsteps; returns the status (NONFINITE/CG_MAXITER/INACTIVE are returned, not raised)."""
        st = _lib.load().gbfem_step(self._h, float(dt), int(nsteps), int(flags))
        self.last_status = st
        if st in raise_on:
            raise GbfemError(st, _lib.last_error(self._h))
        return st

    def stats(self) -> dict:
        s = _lib.Stats()
        _lib.load().gbfem_get_stats(self._h, ctypes.byref(s))
        return s.as_dict()

    def state(self):
        x = np.empty(self.n)
        v = np.empty(self.n)
        self._check(_lib.load().gbfem_get_state(self._h, dptr(x), dptr(v)))
        return x, v

    def set_state(self, x=None, v=None):
        xa = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        va = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        self._check(_lib.load().gbfem_set_state(self._h, dptr(xa) if xa is not None else None,
                                                dptr(va) if va is not None else None))

    def set_velocities(self, dofs, values):
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        values = np.ascontiguousarray(values, dtype=np.float64)
        self._check(_lib.load().gbfem_set_velocities(self._h, dofs.size, iptr(dofs), dptr(values)))

    def device_state(self):
        x, v = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.load().gbfem_device_state(self._h, ctypes.byref(x), ctypes.byref(v))
        return x.value, v.value

    def stream(self):
        s = ctypes.c_void_p()
        _lib.load().gbfem_stream(self._h, ctypes.byref(s))
        return s.value

    def reactivate(self):
        _lib.load().gbfem_reactivate(self._h)

    def pattern(self):
        colptr = np.empty(self.n + 1, dtype=np.int32)
        rowidx = np.empty(self.nnz, dtype=np.int32)
        self._check(_lib.load().gbfem_get_pattern(self._h, iptr(colptr), iptr(rowidx)))
        return colptr, rowidx

    def scatter(self):
        m = np.empty(self.num_tets * (3 * self.nodes_per_element) ** 2, dtype=np.int32)
        self._check(_lib.load().gbfem_get_scatter(self._h, iptr(m)))
        return m

    def system(self):
        S, rhs, f = np.empty(self.nnz), np.empty(self.n), np.empty(self.n)
        self._check(_lib.load().gbfem_get_system(self._h, dptr(S), dptr(rhs), dptr(f)))
        return dict(S=S, rhs=rhs, f=f)


class CgSolver:
    """``LinearSparseSolveAndInverseCG`` on the GPU for a caller CSC matrix."""

    def __init__(self, colptr, rowidx, values, device=0):
        self._colptr = np.ascontiguousarray(colptr, dtype=np.int32)
        self._rowidx = np.ascontiguousarray(rowidx, dtype=np.int32)
        self._vals = np.ascontiguousarray(values, dtype=np.float64)
        self.n = self._colptr.size - 1
        h = ctypes.c_void_p()
        L = _lib.load()
        st = L.gbfem_cg_create(self.n, iptr(self._colptr), iptr(self._rowidx), dptr(self._vals), device,
                               ctypes.byref(h))
        if st != _lib.GBFEM_OK:
            raise GbfemError(st, _lib.last_error(None))
        self._h = h

    def set_tolerance(self, tol):
        _lib.load().gbfem_cg_set_tolerance(self._h, float(tol))

    def set_max_iterations(self, it):
        _lib.load().gbfem_cg_set_max_iterations(self._h, int(it))

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        it = ctypes.c_int32()
        res = ctypes.c_double()
        st = _lib.load().gbfem_cg_solve(self._h, dptr(b), dptr(x), ctypes.byref(it), ctypes.byref(res))
        if st not in (_lib.GBFEM_OK, _lib.GBFEM_CG_MAXITER):
            raise GbfemError(st, "cg solve failed")
        return x, it.value, res.value, st

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().gbfem_cg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
