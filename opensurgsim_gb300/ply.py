"""PLY ingest of OpenSurgSim FEM-3D meshes into a TetMesh.

Reads the element layout that ``Fem3DPlyReaderDelegate`` / ``FemPlyReaderDelegate``
(``Physics/Fem3DPlyReaderDelegate.cpp:30-100``, ``Physics/FemPlyReaderDelegate.cpp:31-191``) consume:

- ``vertex`` with ``x y z``;
- ``3d_element`` with a ``vertex_indices`` list (4 ids per tetrahedron or 8 per hexahedron, the
  counts Fem3DPlyReaderDelegate.cpp:76 accepts; one count per file), optionally carrying its own
  ``mass_density``, ``poisson_ratio`` and ``young_modulus``;
- ``material`` (one row: ``mass_density poisson_ratio young_modulus``) applied to every element that
  carries none;
- ``boundary_condition`` (or ``boundary_conditions``) with ``vertex_index``: every dof of the listed
  vertices is fixed.

Other elements (``face`` and so on) are skipped. ASCII and binary (little/big endian) files are
read.
"""

from __future__ import annotations

import numpy as np

from .mesh import TetMesh

_TYPES = {
    "char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2", "ushort": "u2",
    "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4", "float": "f4", "float32": "f4",
    "double": "f8", "float64": "f8",
}


class PlyError(ValueError):
    pass


def _parse_header(f):
    if f.readline().strip() != b"ply":
        raise PlyError("not a PLY file")
    fmt = None
    elements = []
    while True:
        line = f.readline()
        if not line:
            raise PlyError("unterminated header")
        tok = line.split()
        if not tok or tok[0] in (b"comment", b"obj_info"):
            continue
        if tok[0] == b"format":
            fmt = tok[1].decode()
        elif tok[0] == b"element":
            elements.append({"name": tok[1].decode(), "count": int(tok[2]), "props": []})
        elif tok[0] == b"property":
            if tok[1] == b"list":
                elements[-1]["props"].append((tok[4].decode(), "list", _TYPES[tok[2].decode()], _TYPES[tok[3].decode()]))
            else:
                elements[-1]["props"].append((tok[2].decode(), "scalar", _TYPES[tok[1].decode()], None))
        elif tok[0] == b"end_header":
            break
    if fmt not in ("ascii", "binary_little_endian", "binary_big_endian"):
        raise PlyError(f"unsupported PLY format {fmt}")
    return fmt, elements


def _read_elements(f, fmt, elements):
    data = {}
    if fmt == "ascii":
        words = f.read().split()
        pos = 0
        for el in elements:
            rows = []
            for _ in range(el["count"]):
                row = {}
                for name, kind, t0, t1 in el["props"]:
                    if kind == "list":
                        cnt = int(words[pos])
                        pos += 1
                        row[name] = [float(w) for w in words[pos:pos + cnt]]
                        pos += cnt
                    else:
                        row[name] = float(words[pos])
                        pos += 1
                rows.append(row)
            data[el["name"]] = rows
        return data
    end = "<" if fmt == "binary_little_endian" else ">"
    buf = f.read()
    pos = 0
    for el in elements:
        rows = []
        for _ in range(el["count"]):
            row = {}
            for name, kind, t0, t1 in el["props"]:
                if kind == "list":
                    dt0 = np.dtype(end + t0)
                    cnt = int(np.frombuffer(buf, dt0, 1, pos)[0])
                    pos += dt0.itemsize
                    dt1 = np.dtype(end + t1)
                    row[name] = np.frombuffer(buf, dt1, cnt, pos).astype(float).tolist()
                    pos += cnt * dt1.itemsize
                else:
                    dt = np.dtype(end + t0)
                    row[name] = float(np.frombuffer(buf, dt, 1, pos)[0])
                    pos += dt.itemsize
            rows.append(row)
        data[el["name"]] = rows
    return data


def load_fem3d(path) -> TetMesh:
    """Read a FEM-3D PLY file (the format Fem3DRepresentation::loadFem reads). ``tets`` of the result
    has 4 columns for tetrahedra, 8 for hexahedra (Fem3DElementCube node order)."""
    with open(path, "rb") as f:
        fmt, elements = _parse_header(f)
        data = _read_elements(f, fmt, elements)
    return mesh_from_ply_data(data)


def mesh_from_ply_data(data) -> TetMesh:
    if "vertex" not in data or "3d_element" not in data:
        raise PlyError("missing vertex or 3d_element")
    nodes = np.array([[r["x"], r["y"], r["z"]] for r in data["vertex"]], dtype=np.float64)
    els = data["3d_element"]
    counts = {len(r["vertex_indices"]) for r in els}
    if not counts <= {4, 8}:
        raise PlyError("3d_element vertex counts must be 4 (tetrahedra) or 8 (hexahedra)")
    if len(counts) > 1:
        raise PlyError("a mesh holds one element type: 4- and 8-node 3d_elements are mixed")
    tets = np.array([r["vertex_indices"] for r in els], dtype=np.int64)
    if tets.min() < 0 or tets.max() >= nodes.shape[0]:
        raise PlyError("element refers to a missing vertex")
    mat = (data.get("material") or [None])[0]
    E = np.empty(len(els))
    nu = np.empty(len(els))
    rho = np.empty(len(els))
    for i, r in enumerate(els):
        src = r if "young_modulus" in r else mat
        if src is None:
            raise PlyError("no material for element %d" % i)
        E[i], nu[i], rho[i] = src["young_modulus"], src["poisson_ratio"], src["mass_density"]
    bc_rows = data.get("boundary_condition") or data.get("boundary_conditions") or []
    bc_nodes = [int(r["vertex_index"]) for r in bc_rows]
    bc = np.array([3 * n + k for n in bc_nodes for k in range(3)], dtype=np.int32)
    return TetMesh(nodes, tets.astype(np.int32), E, nu, rho, bc)
