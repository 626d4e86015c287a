"""ctypes binding of the C ABI declared in include/gbfem.h (libgbfem.so, built in-tree).

There is no CPU fallback: if the shared library is missing, importing the bindings raises.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbfem.so")

GBFEM_OK = 0
GBFEM_INVALID_ARG = 1
GBFEM_DEGENERATE_ELEMENT = 2
GBFEM_CG_MAXITER = 3
GBFEM_NONFINITE = 4
GBFEM_CUDA_ERROR = 5
GBFEM_INACTIVE = 6
GBFEM_OUT_OF_MEMORY = 7
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "DEGENERATE_ELEMENT", 3: "CG_MAXITER", 4: "NONFINITE",
                5: "CUDA_ERROR", 6: "INACTIVE", 7: "OUT_OF_MEMORY"}

PRECISION_FP64 = 0
PRECISION_MIXED = 1

ELEMENT_COROTATIONAL_TET = 0
ELEMENT_LINEAR_TET = 1
ELEMENT_HEXAHEDRON = 2

STEP_TIME_PHASES = 1
STEP_KEEP_SYSTEM = 2
STEP_TIME_KERNELS = 4
STEP_GRAPH = 8
COMPLIANCE_WARPING = 1
# CG schedules of the persistent solve (gbfem_get_tuning / gbfem_set_tuning)
CG_TWO_PHASE = 0
CG_FP64 = 1
CG_ONE_PHASE = 2

# Every symbol the header declares; the CPU tests check the library exports all of them.
EXPORTED = [
    "gbfem_params_default", "gbfem_create", "gbfem_destroy", "gbfem_step", "gbfem_get_stats", "gbfem_get_state",
    "gbfem_set_state", "gbfem_set_velocities", "gbfem_set_velocities_device", "gbfem_device_state", "gbfem_stream", "gbfem_reactivate",
    "gbfem_get_sizes", "gbfem_get_pattern", "gbfem_get_scatter", "gbfem_get_system", "gbfem_last_error",
    "gbfem_cg_create", "gbfem_cg_set_tolerance", "gbfem_cg_set_max_iterations", "gbfem_cg_solve",
    "gbfem_cg_destroy", "gbfem_cg_solve_noalloc", "gbfem_batch_create", "gbfem_batch_info",
    "gbfem_batch_segment_stats", "gbfem_set_materials_device", "gbfem_adjoint_step", "gbfem_get_tuning",
    "gbfem_set_tuning", "gbfem_apply_compliance", "gbfem_add_external_force", "gbfem_barrier_selftest",
    "gbfem_set_solver_params", "gbfem_rollout_forward", "gbfem_rollout_backward",
]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("rest_positions", ctypes.POINTER(ctypes.c_double)),
        ("num_tets", ctypes.c_int32),
        ("tets", ctypes.POINTER(ctypes.c_int32)),
        ("young_modulus", ctypes.POINTER(ctypes.c_double)),
        ("poisson_ratio", ctypes.POINTER(ctypes.c_double)),
        ("mass_density", ctypes.POINTER(ctypes.c_double)),
        ("num_bc_dofs", ctypes.c_int32),
        ("bc_dofs", ctypes.POINTER(ctypes.c_int32)),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("rayleigh_mass", ctypes.c_double),
        ("rayleigh_stiffness", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("gravity_enabled", ctypes.c_int32),
        ("newton_max_iterations", ctypes.c_int32),
        ("newton_epsilon", ctypes.c_double),
        ("cg_tolerance", ctypes.c_double),
        ("cg_max_iterations", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("autotune", ctypes.c_int32),
        ("element_type", ctypes.c_int32),
        ("mass_lumping", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 4),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int32),
        ("cg_iterations", ctypes.c_int32),
        ("cg_max_iterations_hit", ctypes.c_int32),
        ("refinement_sweeps", ctypes.c_int32),
        ("cg_relative_residual", ctypes.c_double),
        ("ms_element", ctypes.c_double),
        ("ms_assemble", ctypes.c_double),
        ("ms_solve", ctypes.c_double),
        ("ms_update", ctypes.c_double),
        ("singular_g", ctypes.c_int32),
        ("polar_fallbacks", ctypes.c_int32),
        ("active", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int32),
        ("spmv_timed", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("ms_spmv", ctypes.c_double),
        ("reserved", ctypes.c_double * 2),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


_lib = None


def load():
    """Load libgbfem.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with opensurgsim_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    H, D, I32, I64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32), ctypes.c_int64
    S = ctypes.c_int
    sig = {
        "gbfem_params_default": (S, [ctypes.POINTER(Params)]),
        "gbfem_create": (S, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), ctypes.POINTER(H)]),
        "gbfem_destroy": (S, [H]),
        "gbfem_step": (S, [H, ctypes.c_double, ctypes.c_int32, ctypes.c_uint32]),
        "gbfem_get_stats": (S, [H, ctypes.POINTER(Stats)]),
        "gbfem_get_state": (S, [H, D, D]),
        "gbfem_set_state": (S, [H, D, D]),
        "gbfem_set_velocities": (S, [H, ctypes.c_int32, I32, D]),
        "gbfem_set_velocities_device": (S, [H, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
        "gbfem_device_state": (S, [H, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]),
        "gbfem_stream": (S, [H, ctypes.POINTER(ctypes.c_void_p)]),
        "gbfem_reactivate": (S, [H]),
        "gbfem_get_sizes": (S, [H, ctypes.POINTER(I64), ctypes.POINTER(I64)]),
        "gbfem_get_pattern": (S, [H, I32, I32]),
        "gbfem_get_scatter": (S, [H, I32]),
        "gbfem_get_system": (S, [H, D, D, D]),
        "gbfem_last_error": (S, [H, ctypes.c_char_p, ctypes.c_size_t]),
        "gbfem_cg_create": (S, [ctypes.c_int32, I32, I32, D, ctypes.c_int32, ctypes.POINTER(H)]),
        "gbfem_cg_set_tolerance": (S, [H, ctypes.c_double]),
        "gbfem_cg_set_max_iterations": (S, [H, ctypes.c_int32]),
        "gbfem_cg_solve": (S, [H, D, D, I32, D]),
        "gbfem_cg_destroy": (S, [H]),
        "gbfem_batch_create": (S, [ctypes.c_int32, ctypes.POINTER(MeshDesc), ctypes.POINTER(Params),
                                   ctypes.POINTER(H)]),
        "gbfem_batch_info": (S, [H, I32, I32, I32, ctypes.POINTER(ctypes.c_int64)]),
        "gbfem_batch_segment_stats": (S, [H, I32, I32, I32, D]),
        "gbfem_set_materials_device": (S, [H, ctypes.c_void_p, ctypes.c_void_p]),
        "gbfem_get_tuning": (S, [H, I32, I32, I32, I32]),
        "gbfem_apply_compliance": (S, [H, ctypes.c_int32, D, D, ctypes.c_uint32, I32]),
        "gbfem_set_tuning": (S, [H, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
        "gbfem_set_solver_params": (S, [H, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32]),
        "gbfem_rollout_forward": (S, [H, ctypes.c_double, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 4),
        "gbfem_rollout_backward": (S, [H] + [ctypes.c_void_p] * 6),
        "gbfem_adjoint_step": (S, [H, ctypes.c_double] + [ctypes.c_void_p] * 9 + [ctypes.c_uint32]),
        "gbfem_add_external_force": (S, [H, ctypes.c_int32, D, D, D, D]),
        "gbfem_barrier_selftest": (S, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]),
        "gbfem_cg_solve_noalloc": (S, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                       ctypes.POINTER(ctypes.c_double)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error(handle=None) -> str:
    buf = ctypes.create_string_buffer(1024)
    load().gbfem_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


class GbfemError(RuntimeError):
    """A non-OK gbfem status (the reference's SurgSim::Framework::AssertionFailure equivalent)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"gbfem {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
