"""The OpenSurgSim-named C++ facade (include/surgsim_compat/surgsim_gb300.h) executed on the GPU.

A C++ program written against the facade (tests/support/facade_c1.cpp) is compiled with g++ and
linked against libgbfem.so. It builds a Fem3DRepresentation through the reference's method names,
checks that unsupported integration schemes and linear solvers throw, steps it with update(dt),
then calls OdeSolverEulerImplicit::solve, getSystemMatrix, getComplianceMatrix and
applyCompliance. Everything it writes is compared with the oracle."""

import os
import shutil
import subprocess

import numpy as np
import pytest

from opensurgsim_gb300 import mesh

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def facade_exe(gpu_lib, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ unavailable")
    exe = str(tmp_path_factory.mktemp("facade") / "facade_c1")
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(HERE, "support", "facade_c1.cpp"), "-L" + os.path.join(ROOT, "opensurgsim_gb300"),
                    "-lgbfem", "-Wl,-rpath," + os.path.join(ROOT, "opensurgsim_gb300"), "-o", exe], check=True)
    return exe


def _run(exe, scene, steps, tmp_path):
    m = scene.mesh
    bc_nodes = np.unique(m.bc_dofs // 3).astype(np.int32)
    assert np.array_equal(np.sort(m.bc_dofs), np.sort((3 * bc_nodes[:, None] + np.arange(3)).ravel()))
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        np.array([m.num_nodes, m.num_tets, bc_nodes.size], dtype=np.int32).tofile(f)
        m.nodes.astype(np.float64).tofile(f)
        m.tets.astype(np.int32).tofile(f)
        for a in (m.young, m.poisson, m.density):
            np.asarray(a, dtype=np.float64).tofile(f)
        bc_nodes.tofile(f)
        np.array([scene.rayleigh_mass, scene.rayleigh_stiffness, *scene.gravity, scene.dt, scene.cg_tolerance],
                 dtype=np.float64).tofile(f)
    out = tmp_path / "out.bin"
    res = subprocess.run([exe, str(path), str(out), str(steps)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, (res.returncode, res.stdout, res.stderr)
    raw = out.read_bytes()
    n = m.num_dofs
    off = 0

    def take(count, dtype=np.float64):
        nonlocal off
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a

    r = dict(x=take(n), v=take(n), nx=take(n), nv=take(n))
    nnz = int(take(1, np.int64)[0])
    r["S"] = take(nnz)
    if n <= 600:
        r["C"] = take(n * n).reshape(n, n, order="F")
    r["applied"] = take(2 * n).reshape(n, 2, order="F")
    assert off == len(raw)
    return r


def test_facade_steps_c1_for_100_steps_like_the_oracle(facade_exe, tmp_path):
    """The 10x10x10 cube (5,000 tets), 100 updates through the facade, then one solve: states within
    1e-8 of the oracle's, the system matrix of the solve within 1e-12 (max-norm relative), and
    applyCompliance within 1e-8 of the oracle's."""
    from oracle import oracle as O

    scene = mesh.scene_cube(10, 10, 10)
    r = _run(facade_exe, scene, 100, tmp_path)
    o = O.OracleModel.from_scene(scene)
    assert o.step(scene.dt, 100) == 0
    ox, ov = o.state()
    rest = scene.mesh.nodes.ravel()
    assert rel(r["x"] - rest, ox - rest) <= 1e-8
    assert rel(r["v"], ov) <= 1e-8
    assert o.step(scene.dt, 1) == 0
    nx, nv = o.state()
    assert rel(r["nx"] - rest, nx - rest) <= 1e-8
    assert rel(r["nv"], nv) <= 1e-8
    S = o.system()["S"]
    assert np.max(np.abs(r["S"] - S)) <= 1e-12 * np.max(np.abs(S))
    n = scene.mesh.num_dofs
    b = np.stack([1.0 + 0.001 * np.arange(n), np.where(np.arange(n) % 3 == 2, -1.0, 0.5)], axis=1)
    want, _, _ = o.apply_compliance(b)
    assert rel(r["applied"], want) <= 1e-8


def test_facade_compliance_matrix_on_a_small_body(facade_exe, tmp_path):
    """getComplianceMatrix after solve(..., computeCompliance=true): the dense inverse of the solve's
    system with the boundary rows and columns zeroed (OdeSolver.cpp:69-76), against the oracle's
    compliance of the identity's columns."""
    from oracle import oracle as O

    scene = mesh.scene_cube(2, 2, 3, seed=2)
    r = _run(facade_exe, scene, 5, tmp_path)
    o = O.OracleModel.from_scene(scene)
    assert o.step(scene.dt, 6) == 0
    n = scene.mesh.num_dofs
    want, _, _ = o.apply_compliance(np.eye(n))
    assert rel(r["C"], want) <= 1e-8
    bc = scene.mesh.bc_dofs
    assert np.all(r["C"][bc, :] == 0.0) and np.all(r["C"][:, bc] == 0.0)
