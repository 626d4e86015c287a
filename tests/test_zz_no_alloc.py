"""gbfem_cg_solve_noalloc: the CG solve for callers that must not allocate device memory.

Some callers cannot call cudaMalloc once they are running -- a simulator's fixed-rate physics or
haptics loop, where an allocation can stall at an unpredictable moment, or a host that reserves
all device memory at start-up. The no-allocation entry point works out of a fixed scratch area
inside the library. Through the C ABI, these tests check that two consecutive calls give the same
solutions as the allocating entry point (gbfem_cg_create / gbfem_cg_solve) and as the oracle's CG
(the same iteration count, within 1e-10), that repeated calls leave the device's free memory
unchanged, and that a malformed matrix is rejected before the solve reads through it.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fem_system(nsteps):
    """S (CSC, lower triangle is what CG reads) and rhs of a small cube step, from the oracle."""
    from opensurgsim_gb300 import mesh
    from oracle import oracle as O

    scene = mesh.scene_cube(6, 6, 6)
    model = O.OracleModel.from_scene(scene)
    model.step(scene.dt, nsteps)
    colptr, rowidx = model.pattern()
    sysm = model.system()
    return colptr, rowidx, sysm["S"], sysm["rhs"]


def _symmetric_csr(colptr, rowidx, vals):
    import scipy.sparse as sp

    n = colptr.size - 1
    S = sp.csc_matrix((vals, rowidx, colptr), shape=(n, n))
    L = sp.tril(S)
    A = (L + sp.tril(L, -1).T).tocsr()
    A.sort_indices()
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)


def _entry():
    from opensurgsim_gb300 import _lib

    fn = _lib.load().gbfem_cg_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]
    return fn


def _device_system(torch, rp, ci, va, rhs):
    dev = torch.device("cuda:0")
    d = dict(rp=torch.from_numpy(rp).to(dev), ci=torch.from_numpy(ci).to(dev), va=torch.from_numpy(va).to(dev),
             b=torch.from_numpy(rhs.copy()).to(dev),
             x=torch.full((rhs.size,), float("nan"), dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    return d


def _call(fn, d, n, tol):
    it = ctypes.c_int32(-1)
    res = ctypes.c_double(-1.0)
    st = fn(n, d["rp"].data_ptr(), d["ci"].data_ptr(), d["va"].data_ptr(), d["b"].data_ptr(), d["x"].data_ptr(), tol,
            0, None, ctypes.byref(it), ctypes.byref(res))
    return st, it.value, res.value


def test_noalloc_solve_matches_allocating_solve_and_oracle(gpu_lib):
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300 import _lib
    from opensurgsim_gb300.body import CgSolver
    from oracle import oracle as O

    fn = _entry()
    tol = 1e-10
    for call, nsteps in enumerate((1, 7)):  # two calls in a row, different systems
        colptr, rowidx, vals, rhs = _fem_system(nsteps)
        n = rhs.size
        ref = CgSolver(colptr, rowidx, vals)
        ref.set_tolerance(tol)
        x_ref, it_ref, res_ref, st_ref = ref.solve(rhs)
        assert st_ref == _lib.GBFEM_OK
        ref.close()
        x_orc, it_orc, _, st_orc = O.cg_solve(colptr, rowidx, vals, rhs, tol=tol)
        assert st_orc == 0
        d = _device_system(torch, *_symmetric_csr(colptr, rowidx, vals), rhs)
        st, it, res = _call(fn, d, n, tol)
        assert st == _lib.GBFEM_OK, _lib.last_error(None)
        x = d["x"].cpu().numpy()
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        err_orc = np.linalg.norm(x - x_orc) / np.linalg.norm(x_orc)
        print(f"call {call}: n={n} iterations {it} (allocating: {it_ref}, oracle: {it_orc}), rel diff {err:.2e} "
              f"(oracle {err_orc:.2e})")
        assert err <= 1e-10
        assert err_orc <= 1e-10
        assert it == it_ref == it_orc
        assert res < tol


def test_noalloc_calls_allocate_nothing(gpu_lib):
    """After a first call (which sets up the device's scratch address), further calls leave the
    device's free memory exactly where it was."""
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300 import _lib

    fn = _entry()
    colptr, rowidx, vals, rhs = _fem_system(3)
    d = _device_system(torch, *_symmetric_csr(colptr, rowidx, vals), rhs)
    assert _call(fn, d, rhs.size, 1e-10)[0] == _lib.GBFEM_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(fn, d, rhs.size, 1e-10)[0] == _lib.GBFEM_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_malformed_matrix(gpu_lib):
    """A column index outside [0, n) and a decreasing row pointer come back as GBFEM_INVALID_ARG
    from the device-side check; every array keeps its size, so every read stays in bounds."""
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300 import _lib

    fn = _entry()
    colptr, rowidx, vals, rhs = _fem_system(1)
    rp, ci, va = _symmetric_csr(colptr, rowidx, vals)
    n = rhs.size
    bad_col = ci.copy()
    bad_col[ci.size // 2] = n + 5
    d = _device_system(torch, rp, bad_col, va, rhs)
    st, _, _ = _call(fn, d, n, 1e-10)
    assert st == _lib.GBFEM_INVALID_ARG
    assert "column index" in _lib.last_error(None)
    bad_rp = rp.copy()
    bad_rp[n // 2] = bad_rp[n // 2 + 1] + 1  # rowptr decreases after row n/2 (all values stay within nnz)
    d = _device_system(torch, bad_rp, ci, va, rhs)
    st, _, _ = _call(fn, d, n, 1e-10)
    assert st == _lib.GBFEM_INVALID_ARG
    assert "rowptr" in _lib.last_error(None)
    # A sound call afterwards still works.
    d = _device_system(torch, rp, ci, va, rhs)
    assert _call(fn, d, n, 1e-10)[0] == _lib.GBFEM_OK


def test_noalloc_rejects_oversized_systems(gpu_lib):
    from opensurgsim_gb300 import _lib

    fn = _entry()
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = fn(262145, dummy, dummy, dummy, dummy, dummy, 1e-10, 0, None, None, None)
    assert st == _lib.GBFEM_INVALID_ARG
    assert "exceeds" in _lib.last_error(None)
