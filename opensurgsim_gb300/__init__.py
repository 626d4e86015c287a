"""GB300-native corotational-tetrahedron FEM implicit-Euler step (OpenSurgSim hot path).

The compute path is the in-tree CUDA library ``libgbfem.so`` (sm_103a) behind the C ABI of
``include/gbfem.h``; this package is its Python host side.
"""

from . import mesh  # noqa: F401

__all__ = ["mesh", "Body", "CgSolver"]


def __getattr__(name):
    if name in ("Body", "CgSolver"):
        from . import body

        return getattr(body, name)
    raise AttributeError(name)
