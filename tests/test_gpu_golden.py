"""GPU parity on OpenSurgSim's own test meshes (Tetrahedron.ply, wound_deformable.ply, singleTet.ply,
sharedTet.ply, tripleTet.ply) and the one-cube scene of RenderTestFem3DCorotational.cpp against the
committed FP64 oracle vectors (tests/golden, made by tests/golden/make_fixtures.py)."""

import json
import os

import numpy as np
import pytest

from opensurgsim_gb300 import _lib, mesh
from opensurgsim_gb300.body import Body

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = json.load(open(os.path.join(GOLDEN, f"{name}_mesh.json")))
    g = json.load(open(os.path.join(GOLDEN, f"{name}_oracle.json")))
    m = mesh.TetMesh(np.array(d["nodes"]), np.array(d["tets"], np.int32), np.array(d["young"]),
                     np.array(d["poisson"]), np.array(d["density"]), np.array(d["bc_dofs"], np.int32))
    return m, g


@pytest.mark.parametrize("name", ["tetrahedron", "wound_deformable", "single_tet", "shared_tet", "triple_tet",
                                  "render_cube5"])
@pytest.mark.parametrize("precision,tol", [(_lib.PRECISION_FP64, 1e-9), (_lib.PRECISION_MIXED, 1e-6)])
def test_reference_mesh_steps_match_oracle(gpu_lib, name, precision, tol):
    m, g = load(name)
    st = g["step"]
    body = Body(m, rayleigh_mass=st["rayleigh_mass"], rayleigh_stiffness=st["rayleigh_stiffness"],
                cg_tolerance=st["cg_tolerance"], precision=precision)
    assert body.step(st["dt"], st["steps"]) == _lib.GBFEM_OK
    x, v = body.state()
    x0 = m.nodes.ravel()
    ox, ov = np.array(g["x"]), np.array(g["v"])
    err = np.linalg.norm((x - x0) - (ox - x0)) / np.linalg.norm(ox - x0)
    verr = np.linalg.norm(v - ov) / np.linalg.norm(ov)
    print(f"{name} precision={precision}: rel disp err {err:.2e}, rel vel err {verr:.2e}")
    assert err <= tol and verr <= 10 * tol
