"""Failure detection of the batched solve's grid barrier, without a GPU fault.

The mixed-precision solve is one cooperative launch whose blocks wait for one another at a grid
barrier every phase. Each wait has a wall-time limit, after which the kernel records an error and
returns, and the step reports GBFEM_CUDA_ERROR. gbfem_barrier_selftest runs the same barrier code
with a counter that no arrival can complete (a flag that nothing sets), so every wait must run out;
the tests check the status, the time it took, and that the context is still usable afterwards.
"""

import ctypes

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh

pytestmark = pytest.mark.gpu


def _selftest(L, phases, stall, timeout_ns):
    passed = ctypes.c_int32(-1)
    waited = ctypes.c_int64(-1)
    st = L.gbfem_barrier_selftest(phases, stall, timeout_ns, ctypes.byref(passed), ctypes.byref(waited))
    return st, passed.value, waited.value


def test_barrier_passes_every_phase(gpu_lib):
    st, passed, waited = _selftest(gpu_lib, 500, 0, 1_000_000_000)
    assert st == _lib.GBFEM_OK, _lib.last_error()
    assert passed == 500
    assert 0 < waited < 1_000_000_000


@pytest.mark.parametrize("timeout_ns", [2_000_000, 50_000_000])
def test_stalled_barrier_times_out_with_an_error_status(gpu_lib, timeout_ns):
    st, passed, waited = _selftest(gpu_lib, 4, 1, timeout_ns)
    assert st == _lib.GBFEM_CUDA_ERROR
    assert "ran out" in _lib.last_error()
    assert passed == 0
    # The slowest block waited its whole limit, and no block waited much longer.
    assert timeout_ns <= waited < timeout_ns + 200_000_000, waited


def test_context_usable_after_a_timeout(gpu_lib):
    from opensurgsim_gb300.body import Body

    assert _selftest(gpu_lib, 2, 1, 5_000_000)[0] == _lib.GBFEM_CUDA_ERROR
    st, passed, _ = _selftest(gpu_lib, 50, 0, 1_000_000_000)
    assert st == _lib.GBFEM_OK and passed == 50
    # A mixed-precision batch solve (the persistent launch behind the barrier) still steps.
    scenes = [mesh.scene_cube(2, 2, 3, seed=s) for s in range(3)]
    b = Body([s.mesh for s in scenes], precision=_lib.PRECISION_MIXED, cg_tolerance=1e-8,
             gravity=(0, 0, -9.81))
    assert b.step(1e-3, 2) == _lib.GBFEM_OK
    x, v = b.state()
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(v))


def test_selftest_arguments(gpu_lib):
    assert _selftest(gpu_lib, 0, 0, 1_000_000)[0] == _lib.GBFEM_INVALID_ARG
    assert _selftest(gpu_lib, 1, 1, 100)[0] == _lib.GBFEM_INVALID_ARG
    assert _selftest(gpu_lib, 1, 1, 3_000_000_000)[0] == _lib.GBFEM_INVALID_ARG
