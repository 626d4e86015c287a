"""gbfem_cg_solve_noalloc: the CG solve for callers that must not allocate device memory.

Some callers cannot call cudaMalloc once they are running -- a simulator's fixed-rate physics or
haptics loop, where an allocation can stall at an unpredictable moment, or a host that reserves
all device memory at start-up. The no-allocation entry point works out of a fixed scratch area
inside the library; this test checks, through the C ABI, that two consecutive calls give the same
solutions as the allocating entry point (gbfem_cg_create / gbfem_cg_solve), within 1e-10.
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


def test_noalloc_solve_matches_allocating_solve(gpu_lib):
    torch = pytest.importorskip("torch")
    from opensurgsim_gb300 import _lib
    from opensurgsim_gb300.body import CgSolver

    L = _lib.load()
    fn = L.gbfem_cg_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]
    tol = 1e-10
    dev = torch.device("cuda:0")
    for call, nsteps in enumerate((1, 7)):  # two calls in a row, different systems
        colptr, rowidx, vals, rhs = _fem_system(nsteps)
        n = rhs.size
        ref = CgSolver(colptr, rowidx, vals)
        ref.set_tolerance(tol)
        x_ref, it_ref, res_ref, st_ref = ref.solve(rhs)
        assert st_ref == _lib.GBFEM_OK
        rp, ci, va = _symmetric_csr(colptr, rowidx, vals)
        d_rp = torch.from_numpy(rp).to(dev)
        d_ci = torch.from_numpy(ci).to(dev)
        d_va = torch.from_numpy(va).to(dev)
        d_b = torch.from_numpy(rhs.copy()).to(dev)
        d_x = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        it = ctypes.c_int32(-1)
        res = ctypes.c_double(-1.0)
        st = fn(n, d_rp.data_ptr(), d_ci.data_ptr(), d_va.data_ptr(), d_b.data_ptr(), d_x.data_ptr(), tol, 0, None,
                ctypes.byref(it), ctypes.byref(res))
        assert st == _lib.GBFEM_OK, _lib.last_error(None)
        x = d_x.cpu().numpy()
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        print(f"call {call}: n={n} iterations {it.value} (allocating: {it_ref}), rel diff {err:.2e}")
        assert err <= 1e-10
        assert it.value == it_ref
        assert res.value < tol
        ref.close()


def test_noalloc_rejects_oversized_systems(gpu_lib):
    from opensurgsim_gb300 import _lib

    L = _lib.load()
    fn = L.gbfem_cg_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = fn(262145, dummy, dummy, dummy, dummy, dummy, 1e-10, 0, None, None, None)
    assert st == _lib.GBFEM_INVALID_ARG
    assert "exceeds" in _lib.last_error(None)
