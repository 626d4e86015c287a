"""Synthetic meshes, scenes and the PLY ingest (CPU)."""

import json
import os

import numpy as np
import pytest

from opensurgsim_gb300 import mesh, ply

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 3, 4), (10, 10, 10), (20, 20, 40)])
def test_cube_grid_counts_orientation_conformity(dims):
    a, b, c = dims
    nodes, tets = mesh.cube_grid(a, b, c, h=0.01, seed=0)
    assert nodes.shape == ((a + 1) * (b + 1) * (c + 1), 3)
    assert tets.shape == (5 * a * b * c, 4)
    assert mesh.signed_volumes(nodes, tets).min() > 0  # Fem3DElementTetrahedron.cpp:114 never warns
    faces = np.sort(np.concatenate([tets[:, [0, 1, 2]], tets[:, [0, 1, 3]], tets[:, [0, 2, 3]], tets[:, [1, 2, 3]]]),
                    axis=1)
    _, counts = np.unique(faces, axis=0, return_counts=True)
    assert counts.max() == 2  # conforming: every interior triangle is shared by exactly two tets
    assert (counts == 1).sum() == 4 * (a * b + b * c + a * c)  # boundary triangles


def test_node_numbering_and_jitter():
    nodes, _ = mesh.cube_grid(3, 4, 5, h=0.01, jitter=0.1, seed=2)
    exact, _ = mesh.cube_grid(3, 4, 5, h=0.01, jitter=0.0)
    i, j, k = 1, 2, 3
    assert np.allclose(exact[mesh.node_id(i, j, k, 4, 5)], [0.01, 0.02, 0.03])
    d = np.abs(nodes - exact)
    assert d.max() <= 0.1 * 0.01 + 1e-15
    boundary = (exact[:, 0] == 0) | (exact[:, 0] == 0.03) | (exact[:, 1] == 0) | (exact[:, 1] == 0.04) | \
               (exact[:, 2] == 0) | (exact[:, 2] == 0.05)
    assert np.all(d[boundary] == 0)


def test_benchmark_scene_sizes():
    s = mesh.scene_cube(10, 10, 10)
    assert s.mesh.num_tets == 5000 and s.mesh.num_nodes == 1331 and s.mesh.bc_dofs.size == 363
    bar = mesh.scene_bar_compression(a=4, b=4, c=16)
    assert bar.mesh.num_tets == 5 * 4 * 4 * 16
    assert bar.driven_dofs.size == 3 * 25
    v0, v60 = bar.driven_values(0), bar.driven_values(60)
    assert np.allclose(v0[2::3], -0.2 * 16 * bar.mesh.h / (50 * 1e-3)) and np.all(v0[0::3] == 0)
    assert np.all(v60 == 0)
    assert set(bar.driven_dofs) <= set(bar.mesh.bc_dofs)
    assert 0.40 <= bar.mesh.poisson.min() and bar.mesh.poisson.max() <= 0.49
    assert 1e4 <= bar.mesh.young.min() and bar.mesh.young.max() <= 1e6


def test_batch_dims_log_uniform():
    dims = mesh.batch_dims(256, 500, 50000, seed=3)
    nodes = np.array([(a + 1) * (b + 1) * (c + 1) for a, b, c in dims])
    assert len(dims) == 256 and nodes.min() >= 200 and nodes.max() <= 80000
    assert 0.2 < np.mean(np.log(nodes) < np.log(5000)) < 0.8


def _write_ascii(path, m, material_per_element=False):
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\ncomment test\n")
        f.write(f"element vertex {m.num_nodes}\nproperty double x\nproperty double y\nproperty double z\n")
        f.write("element face 1\nproperty list uchar uint vertex_indices\n")
        f.write(f"element 3d_element {m.num_tets}\nproperty list uint uint vertex_indices\n")
        if material_per_element:
            f.write("property double mass_density\nproperty double poisson_ratio\nproperty double young_modulus\n")
        else:
            f.write("element material 1\nproperty double mass_density\nproperty double poisson_ratio\n"
                    "property double young_modulus\n")
        f.write(f"element boundary_condition {m.bc_dofs.size // 3}\nproperty uint vertex_index\nend_header\n")
        for p in m.nodes:
            f.write("%.17g %.17g %.17g\n" % tuple(p))
        f.write("3 0 1 2\n")
        for e, t in enumerate(m.tets):
            extra = " %.17g %.17g %.17g" % (m.density[e], m.poisson[e], m.young[e]) if material_per_element else ""
            f.write("%d %s%s\n" % (len(t), " ".join(str(int(i)) for i in t), extra))
        if not material_per_element:
            f.write("%.17g %.17g %.17g\n" % (m.density[0], m.poisson[0], m.young[0]))
        for n in m.bc_dofs[::3] // 3:
            f.write("%d\n" % n)


def _write_binary(path, m):
    with open(path, "wb") as f:
        hdr = ("ply\nformat binary_little_endian 1.0\n"
               f"element vertex {m.num_nodes}\nproperty double x\nproperty double y\nproperty double z\n"
               f"element 3d_element {m.num_tets}\nproperty list uchar int vertex_indices\n"
               "element material 1\nproperty double mass_density\nproperty double poisson_ratio\n"
               "property double young_modulus\n"
               f"element boundary_condition {m.bc_dofs.size // 3}\nproperty uint vertex_index\nend_header\n")
        f.write(hdr.encode())
        f.write(m.nodes.astype("<f8").tobytes())
        for t in m.tets:
            f.write(np.uint8(4).tobytes() + t.astype("<i4").tobytes())
        f.write(np.array([m.density[0], m.poisson[0], m.young[0]], "<f8").tobytes())
        f.write((m.bc_dofs[::3] // 3).astype("<u4").tobytes())


@pytest.mark.parametrize("kind", ["ascii", "ascii_per_element", "binary"])
def test_ply_roundtrip(tmp_path, kind):
    m = mesh.scene_cube(2, 2, 3).mesh
    if kind == "ascii_per_element":
        m.young = np.linspace(1e4, 1e6, m.num_tets)
    path = tmp_path / "m.ply"
    if kind == "binary":
        _write_binary(path, m)
    else:
        _write_ascii(path, m, material_per_element=(kind == "ascii_per_element"))
    r = ply.load_fem3d(path)
    assert np.allclose(r.nodes, m.nodes, rtol=0, atol=0)
    assert np.array_equal(r.tets, m.tets) and np.array_equal(r.bc_dofs, m.bc_dofs)
    assert np.allclose(r.young, m.young) and np.allclose(r.poisson, m.poisson) and np.allclose(r.density, m.density)


def test_ply_hexahedra(tmp_path):
    from oracle import oracle as O

    m = mesh.scene_divisible_cube(3).mesh
    path = tmp_path / "hex.ply"
    _write_ascii(path, m)
    r = ply.load_fem3d(path)
    assert r.tets.shape == (8, 8) and np.array_equal(r.tets, m.tets)
    assert np.array_equal(r.bc_dofs, m.bc_dofs) and np.allclose(r.young, 15.3e3)
    o = O.OracleModel(r, element_type=2)
    assert o.mass_per_node().sum() == pytest.approx(980.0 * 6.0 ** 3)


def test_ply_rejects_bad_files(tmp_path):
    bad = tmp_path / "bad.ply"
    bad.write_text("ply\nformat ascii 1.0\nelement vertex 1\nproperty double x\nproperty double y\n"
                   "property double z\nelement 3d_element 1\nproperty list uint uint vertex_indices\nend_header\n"
                   "0 0 0\n3 0 0 0\n")
    with pytest.raises(ply.PlyError):
        ply.load_fem3d(bad)
    (tmp_path / "x.ply").write_text("not a ply\n")
    with pytest.raises(ply.PlyError):
        ply.load_fem3d(tmp_path / "x.ply")


@pytest.mark.parametrize("name,counts", [("tetrahedron", (26, 44, 4)), ("wound_deformable", (391, 1476, 79)),
                                         ("single_tet", (4, 1, 1)), ("shared_tet", (7, 2, 1)), ("triple_tet", (10, 3, 1)),
                                         ("render_cube5", (8, 5, 2))])
def test_golden_meshes_from_the_reference(name, counts):
    d = json.load(open(os.path.join(GOLDEN, f"{name}_mesh.json")))
    assert (len(d["nodes"]), len(d["tets"]), len(d["bc_dofs"]) // 3) == counts


@pytest.mark.parametrize("name", ["tetrahedron", "single_tet", "shared_tet", "triple_tet", "render_cube5"])
def test_golden_oracle_vectors_reproduce(name):
    """The committed oracle vectors are what the oracle computes now (pins the oracle itself)."""
    from oracle import oracle as O

    d = json.load(open(os.path.join(GOLDEN, f"{name}_mesh.json")))
    g = json.load(open(os.path.join(GOLDEN, f"{name}_oracle.json")))
    m = mesh.TetMesh(np.array(d["nodes"]), np.array(d["tets"], np.int32), np.array(d["young"]),
                     np.array(d["poisson"]), np.array(d["density"]), np.array(d["bc_dofs"], np.int32))
    st = g["step"]
    model = O.OracleModel(m, rayleigh_mass=st["rayleigh_mass"], rayleigh_stiffness=st["rayleigh_stiffness"],
                          cg_tolerance=st["cg_tolerance"])
    model.step(st["dt"], st["steps"])
    x, v = model.state()
    assert np.array_equal(x, np.array(g["x"])) and np.array_equal(v, np.array(g["v"]))
