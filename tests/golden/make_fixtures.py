"""Regenerate the golden fixtures in this folder (run where the OpenSurgSim tree is available).

- ``<name>_mesh.json``: meshes converted from OpenSurgSim's own PLY test data (vertices, tets,
  material, boundary-condition vertices), read with opensurgsim_gb300.ply;
- ``<name>_oracle.json``: FP64 oracle state (positions, velocities) after a few implicit-Euler
  steps of that mesh, the vectors the GPU parity tests compare against.

Usage: python tests/golden/make_fixtures.py /root/reference
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
}
# Step settings for the oracle vectors: dt, steps, Rayleigh, CG tolerance, gravity (the reference
# default (0, -9.81, 0)).
STEP = dict(dt=1e-3, steps=10, rayleigh_mass=0.01, rayleigh_stiffness=0.001, cg_tolerance=1e-12)


def main(ref_root):
    from oracle import oracle as O

    for name, rel in SOURCES.items():
        m = ply.load_fem3d(os.path.join(ref_root, rel))
        mesh_json = dict(nodes=m.nodes.tolist(), tets=m.tets.tolist(), young=m.young.tolist(),
                         poisson=m.poisson.tolist(), density=m.density.tolist(), bc_dofs=m.bc_dofs.tolist(),
                         source=rel)
        with open(os.path.join(HERE, f"{name}_mesh.json"), "w") as f:
            json.dump(mesh_json, f)
        model = O.OracleModel(m, rayleigh_mass=STEP["rayleigh_mass"], rayleigh_stiffness=STEP["rayleigh_stiffness"],
                              cg_tolerance=STEP["cg_tolerance"])
        st = model.step(STEP["dt"], STEP["steps"])
        x, v = model.state()
        with open(os.path.join(HERE, f"{name}_oracle.json"), "w") as f:
            json.dump(dict(step=STEP, status=st, x=x.tolist(), v=v.tolist()), f)
        print(name, m.num_nodes, "nodes", m.num_tets, "tets", m.bc_dofs.size // 3, "BC nodes, oracle status", st)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
