"""Regenerate the golden fixtures in this folder (run where the OpenSurgSim tree is available).

- ``<name>_mesh.json``: meshes converted from OpenSurgSim's own PLY test data (vertices, tets,
  material, boundary-condition vertices), read with opensurgsim_gb300.ply;
- ``<name>_oracle.json``: FP64 oracle state (positions, velocities) after a few implicit-Euler
  steps of that mesh, the vectors the GPU parity tests compare against.
- ``render_cube5``: the scene of RenderTestFem3DCorotational.cpp:46-98 -- one unit cube centred on
  the origin (corner id = dx + 2 dy + 4 dz), split into the same 5 corotational tetrahedra as
  ``mesh.cube_grid``'s even cubes, rho 8000, nu 0.45, E 1e6, Rayleigh 1e-2 / 1e-3, nodes 0 and 1 fixed.

Usage: python tests/golden/make_fixtures.py <path of the OpenSurgSim source tree>
"""

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from opensurgsim_gb300 import ply  # noqa: E402

SOURCES = {
    "tetrahedron": "SurgSim/Physics/UnitTests/Data/PlyReaderTests/Tetrahedron.ply",
    "wound_deformable": "SurgSim/Testing/Data/Geometry/wound_deformable.ply",
    "single_tet": "SurgSim/Physics/UnitTests/Data/singleTet.ply",
    "shared_tet": "SurgSim/Physics/UnitTests/Data/sharedTet.ply",
    "triple_tet": "SurgSim/Physics/UnitTests/Data/tripleTet.ply",
}
# Step settings for the oracle vectors: dt, steps, Rayleigh, CG tolerance, gravity (the reference
# default (0, -9.81, 0)).
STEP = dict(dt=1e-3, steps=10, rayleigh_mass=0.01, rayleigh_stiffness=0.001, cg_tolerance=1e-12)


def render_cube5():
    import numpy as np

    from opensurgsim_gb300 import mesh

    nodes = np.array([[(q & 1) - 0.5, ((q >> 1) & 1) - 0.5, ((q >> 2) & 1) - 0.5] for q in range(8)])
    tets = mesh._SPLIT_EVEN.astype(np.int32)
    bc = np.arange(6, dtype=np.int32)  # all dofs of nodes 0 and 1
    return mesh.TetMesh(nodes, tets, np.full(5, 1e6), np.full(5, 0.45), np.full(5, 8000.0), bc)


def main(ref_root):
    from oracle import oracle as O

    items = [(name, rel, ply.load_fem3d(os.path.join(ref_root, rel)), STEP) for name, rel in SOURCES.items()]
    items.append(("render_cube5", "SurgSim/Physics/RenderTests/RenderTestFem3DCorotational.cpp:46-98", render_cube5(),
                  dict(STEP, rayleigh_mass=1e-2, rayleigh_stiffness=1e-3, steps=100)))
    for name, rel, m, step in items:
        mesh_json = dict(nodes=m.nodes.tolist(), tets=m.tets.tolist(), young=m.young.tolist(),
                         poisson=m.poisson.tolist(), density=m.density.tolist(), bc_dofs=m.bc_dofs.tolist(),
                         source=rel)
        with open(os.path.join(HERE, f"{name}_mesh.json"), "w") as f:
            json.dump(mesh_json, f)
        model = O.OracleModel(m, rayleigh_mass=step["rayleigh_mass"], rayleigh_stiffness=step["rayleigh_stiffness"],
                              cg_tolerance=step["cg_tolerance"])
        st = model.step(step["dt"], step["steps"])
        x, v = model.state()
        with open(os.path.join(HERE, f"{name}_oracle.json"), "w") as f:
            json.dump(dict(step=step, status=st, x=x.tolist(), v=v.tolist()), f)
        print(name, m.num_nodes, "nodes", m.num_tets, "tets", m.bc_dofs.size // 3, "BC nodes, oracle status", st)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the OpenSurgSim source tree>")
    main(sys.argv[1])
