"""CPU model of the persistent solve's two CG schedules (gbfem_pcg.cu), in numpy float32 with the
kernel's reliable-update rule: the FP32 iteration works on the residual scaled by s = |r_true|, a
refresh recomputes the true residual b - A x in FP64 whenever |r|^2 has dropped by `drop` since the
last refresh (or the FP32 residual says converged), convergence is decided on that true residual at
Eigen's |r|^2 < tol^2 |b|^2, and the search direction is kept (rescaled) across a refresh.

- two-phase: the textbook PCG recurrences (SpMV q = A p with p.q; then x, r, z and r.z);
- one-phase: Chronopoulos and Gear's recurrences (s = A p kept by recurrence, the SpMV w = A u on the
  preconditioned residual, r.u and w.u from one reduction), including the rescale phase after a
  refresh that recomputes w = A u and scales p and s.

The systems are the ones the oracle assembles for a stepped body (S with the boundary conditions
applied, symmetric from its lower triangle). The two schedules must need the same iterations within a
tenth and reach the FP64 direct solution to the same accuracy; this is what licenses the autotuner
to pick either."""

import math

import numpy as np
import pytest

f32 = np.float32


def _system(a, b, c, young, steps=3, seed=0):
    import scipy.sparse as sp

    from opensurgsim_gb300 import mesh
    from oracle import oracle as O

    scene = mesh.scene_cube(a, b, c, seed=seed, young=young)
    model = O.OracleModel.from_scene(scene)
    model.step(scene.dt, steps)
    colptr, rowidx = model.pattern()
    S = model.system()
    n = colptr.size - 1
    A = sp.csc_matrix((S["S"], rowidx, colptr), shape=(n, n))
    L = sp.tril(A)
    A = (L + sp.tril(L, -1).T).tocsr()
    A.sort_indices()
    A32 = A.astype(f32)
    return A32, A32.astype(np.float64), S["rhs"]


def _jacobi(A32):
    d = A32.diagonal().astype(np.float64)
    return np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 1.0).astype(f32)


def _dot(a, b):
    return float(np.dot(a.astype(np.float64), b.astype(np.float64)))


def two_phase(A32, A64, b, tol=1e-10, drop=1e5):
    n = b.size
    cap = 2 * n + 64
    inv = _jacobi(A32)
    thr = max(tol * tol * (b @ b), np.finfo(float).tiny)
    s = math.sqrt(b @ b)
    r = (b / s).astype(f32)
    z = inv * r
    rz, rr_last = _dot(r, z), _dot(r, r)
    p = np.zeros(n, f32)
    x, xd = np.zeros(n), np.zeros(n, f32)
    beta, it, refreshes = 0.0, 0, 0
    while True:
        p = (z + f32(beta) * p).astype(f32)
        q = (A32 @ p).astype(f32)
        alpha = rz / _dot(p, q)
        xd = (xd + f32(alpha * s) * p).astype(f32)
        r = (r - f32(alpha) * q).astype(f32)
        z = inv * r
        rr, rz_new = _dot(r, r), _dot(r, z)
        if s * s * rr < thr or rr < rr_last / drop or it + 1 >= cap:
            x, xd = x + xd.astype(np.float64), np.zeros(n, f32)
            r64 = b - A64 @ x
            refreshes += 1
            if r64 @ r64 < thr or it + 1 >= cap:
                return x, it, refreshes
            s_new = math.sqrt(r64 @ r64)
            ratio, s = s / s_new, s_new
            r = (r64 / s).astype(f32)
            z = inv * r
            p = (p * f32(ratio)).astype(f32)
            rz_new = _dot(r, z)
            beta, rz, rr_last = rz_new / (rz * ratio * ratio), rz_new, _dot(r, r)
        else:
            beta, rz = rz_new / rz, rz_new
        it += 1


def one_phase(A32, A64, b, tol=1e-10, drop=1e5):
    n = b.size
    cap = 2 * n + 64
    inv = _jacobi(A32)
    thr = max(tol * tol * (b @ b), np.finfo(float).tiny)
    s = math.sqrt(b @ b)
    # The first phase is the rescale phase with no refresh before it: beta = 0, alpha = r.u / w.u.
    r = (b / s).astype(f32)
    u = inv * r
    w = (A32 @ u).astype(f32)
    gam = _dot(r, u)
    alpha, beta, rr_last = gam / _dot(w, u), 0.0, _dot(r, r)
    p, sv = np.zeros(n, f32), np.zeros(n, f32)
    x, xd = np.zeros(n), np.zeros(n, f32)
    it, refreshes = 0, 0
    while True:
        # One phase: p_k, s_k, x, r_{k+1}, u_{k+1} and the SpMV w_{k+1} = A u_{k+1}; r.u, w.u, |r|^2.
        p = (u + f32(beta) * p).astype(f32)
        sv = (w + f32(beta) * sv).astype(f32)
        xd = (xd + f32(alpha * s) * p).astype(f32)
        r = (r - f32(alpha) * sv).astype(f32)
        u = inv * r
        w = (A32 @ u).astype(f32)
        g_new, d_new, rr = _dot(r, u), _dot(w, u), _dot(r, r)
        if s * s * rr < thr or rr < rr_last / drop or it + 1 >= cap:
            # Residual phase, then the rescale phase (w = A u again, p and s rescaled).
            x, xd = x + xd.astype(np.float64), np.zeros(n, f32)
            r64 = b - A64 @ x
            refreshes += 1
            if r64 @ r64 < thr or it + 1 >= cap:
                return x, it, refreshes
            s_new = math.sqrt(r64 @ r64)
            ratio, s = s / s_new, s_new
            r = (r64 / s).astype(f32)
            u = inv * r
            w = (A32 @ u).astype(f32)
            p, sv = (p * f32(ratio)).astype(f32), (sv * f32(ratio)).astype(f32)
            g_new, d_new = _dot(r, u), _dot(w, u)
            beta = g_new / (gam * ratio * ratio)
            rr_last = _dot(r, r)
        else:
            beta = g_new / gam
        alpha = g_new / (d_new - beta * g_new / alpha)
        gam = g_new
        it += 1


@pytest.mark.parametrize("dims,young", [((4, 4, 5), 1e4), ((5, 5, 6), 2e5), ((3, 6, 4), 8e5)])
def test_one_phase_matches_two_phase(dims, young):
    import scipy.sparse.linalg as spla

    A32, A64, b = _system(*dims, young)
    x_ref = spla.spsolve(A64.tocsc(), b)
    x2, it2, rf2 = two_phase(A32, A64, b)
    x1, it1, rf1 = one_phase(A32, A64, b)
    e2 = np.linalg.norm(x2 - x_ref) / np.linalg.norm(x_ref)
    e1 = np.linalg.norm(x1 - x_ref) / np.linalg.norm(x_ref)
    print(f"{dims} E {young:g}: two-phase {it2} iterations, {rf2} refreshes, err {e2:.1e}; "
          f"one-phase {it1}, {rf1}, err {e1:.1e}")
    # Within 10%: on the stiff small system (141 iterations for 420 dofs, where FP32 CG drifts from
    # conjugacy) the one-phase recurrences needed 151; on the others the counts agree to one.
    assert abs(it1 - it2) <= max(3, it2 // 10)
    assert e1 < 1e-8 and e2 < 1e-8
    # Both stop on the same FP64 residual rule.
    for x in (x1, x2):
        r = b - A64 @ x
        assert r @ r < (1e-10) ** 2 * (b @ b)
