"""The C ABI: the library builds, loads and exports every symbol include/gbfem.h declares; host-side
argument validation works without a GPU; the C++ facade compiles (CPU)."""

import ctypes
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbfem.h")


@pytest.fixture(scope="module")
def lib():
    from opensurgsim_gb300 import build, _lib

    build.build()
    return _lib.load()


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GBFEM_API\s+gbfem_status\s+(gbfem_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    from opensurgsim_gb300 import _lib

    decl = declared_symbols()
    assert len(decl) >= 20
    assert sorted(_lib.EXPORTED) == decl
    for name in decl:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gbfem_\w+)", out))
    assert set(decl) <= exported
    assert exported <= set(decl), "library exports undeclared symbols: %s" % (exported - set(decl))


def test_header_constants_match_the_python_bindings():
    """The #define'd flags and CG schedules of gbfem.h have the values the ctypes layer (and
    bench.py's schedule names) use."""
    from opensurgsim_gb300 import _lib

    import bench

    text = open(HEADER).read()
    defines = {k: int(v) for k, v in re.findall(r"#define\s+GBFEM_(\w+)\s+(\d+)u?\b", text)}
    for name in ("CG_TWO_PHASE", "CG_ONE_PHASE", "CG_FP64", "STEP_GRAPH", "STEP_TIME_KERNELS", "STEP_KEEP_SYSTEM",
                 "STEP_TIME_PHASES", "ELEMENT_COROTATIONAL_TET", "ELEMENT_LINEAR_TET", "ELEMENT_HEXAHEDRON"):
        assert defines[name] == getattr(_lib, name), name
    assert {defines[k] for k in defines if k.startswith("CG_")} == set(bench.SCHEDULE_NAMES)
    assert bench.SCHEDULE_NAMES[_lib.CG_ONE_PHASE] == "one-phase"
    assert bench.vector_passes(_lib.CG_ONE_PHASE) == 11 and bench.vector_passes(_lib.CG_TWO_PHASE) == 10


def test_params_default(lib):
    from opensurgsim_gb300 import _lib

    p = _lib.Params()
    assert lib.gbfem_params_default(ctypes.byref(p)) == 0
    assert tuple(p.gravity) == (0.0, -9.81, 0.0)  # Representation.cpp:36
    assert p.newton_max_iterations == 1 and p.newton_epsilon == 1e-5  # OdeSolverEulerImplicit.cpp:26
    assert p.cg_tolerance == np.finfo(float).eps and p.cg_max_iterations == 0  # Eigen defaults


def _desc(m, npe=4):
    from opensurgsim_gb300 import _lib

    keep = [np.ascontiguousarray(m.nodes, np.float64).ravel(), np.ascontiguousarray(m.tets, np.int32).ravel(),
            np.ascontiguousarray(m.young, np.float64), np.ascontiguousarray(m.poisson, np.float64),
            np.ascontiguousarray(m.density, np.float64), np.ascontiguousarray(m.bc_dofs, np.int32)]
    d = _lib.MeshDesc(keep[0].size // 3, _lib.dptr(keep[0]), keep[1].size // npe, _lib.iptr(keep[1]),
                      _lib.dptr(keep[2]), _lib.dptr(keep[3]), _lib.dptr(keep[4]), keep[5].size,
                      _lib.iptr(keep[5]) if keep[5].size else None)
    return d, keep


def _create_hex(lib, m):
    from opensurgsim_gb300 import _lib

    d, keep = _desc(m, npe=8)
    p = _lib.Params()
    lib.gbfem_params_default(ctypes.byref(p))
    p.element_type = _lib.ELEMENT_HEXAHEDRON
    h = ctypes.c_void_p()
    st = lib.gbfem_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
    if h.value:
        lib.gbfem_destroy(h)
    return st


def test_hexahedron_orderings_checked_on_the_host(lib):
    """Fem3DElementCubeTests.cpp NodeOrderingTest / VolumeTest cases through gbfem_create: the
    orderings the reference's initialize rejects fail with DEGENERATE_ELEMENT before any device
    work; the accepted ones pass the host checks (and then need a GPU)."""
    from opensurgsim_gb300 import _lib, mesh
    from test_oracle_hex import NODE_IDS, POINTS, hex_orderings

    for ids, bad in hex_orderings():
        m = mesh.TetMesh(POINTS.copy(), np.array([ids], np.int32), np.array([1e6]), np.array([0.45]),
                         np.array([1000.0]), np.zeros(0, np.int32))
        st = _create_hex(lib, m)
        if bad:
            assert st == _lib.GBFEM_DEGENERATE_ELEMENT, ids
        else:
            assert st in (_lib.GBFEM_OK, _lib.GBFEM_CUDA_ERROR), ids
    flat = POINTS.copy()
    flat[4:] = flat[:4]
    m = mesh.TetMesh(flat, np.array([NODE_IDS], np.int32), np.array([1e6]), np.array([0.45]), np.array([1000.0]),
                     np.zeros(0, np.int32))
    assert _create_hex(lib, m) == _lib.GBFEM_DEGENERATE_ELEMENT
    rep = list(NODE_IDS)
    rep[5] = rep[0]
    m.nodes = POINTS.copy()
    m.tets = np.array([rep], np.int32)
    assert _create_hex(lib, m) == _lib.GBFEM_INVALID_ARG


@pytest.mark.parametrize("bad", ["node", "material", "bc", "nu", "repeat", "empty"])
def test_create_rejects_invalid_input_on_the_host(lib, bad):
    from opensurgsim_gb300 import _lib, mesh

    m = mesh.scene_cube(2, 2, 2).mesh
    if bad == "node":
        m.tets[3, 1] = m.num_nodes
    elif bad == "material":
        m.young[2] = -1.0
    elif bad == "bc":
        m.bc_dofs[0] = 3 * m.num_nodes
    elif bad == "nu":
        m.poisson[0] = 0.5  # FemElement.cpp:38-39: 0 < nu < 0.5
    elif bad == "repeat":
        m.tets[0, 1] = m.tets[0, 0]
    d, keep = _desc(m)
    if bad == "empty":
        d.num_tets = 0
    p = _lib.Params()
    lib.gbfem_params_default(ctypes.byref(p))
    h = ctypes.c_void_p()
    st = lib.gbfem_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
    if bad == "repeat":
        # repeated nodes are caught after the device is opened; without a GPU that step fails first
        assert st in (_lib.GBFEM_INVALID_ARG, _lib.GBFEM_CUDA_ERROR)
    else:
        assert st == _lib.GBFEM_INVALID_ARG
        assert _lib.last_error(None)
    assert not h.value


def test_create_without_gpu_fails_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from opensurgsim_gb300 import _lib, mesh

    d, keep = _desc(mesh.scene_cube(2, 2, 2).mesh)
    p = _lib.Params()
    lib.gbfem_params_default(ctypes.byref(p))
    h = ctypes.c_void_p()
    assert lib.gbfem_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h)) == _lib.GBFEM_CUDA_ERROR
    assert "CUDA" in _lib.last_error(None)


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from opensurgsim_gb300 import _lib

    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    st = lib.gbfem_cg_solve_noalloc(262145, dummy, dummy, dummy, dummy, dummy, 1e-10, 0, None, None, None)
    assert st == _lib.GBFEM_INVALID_ARG
    assert "exceeds" in _lib.last_error(None)


def test_barrier_selftest_validates_its_arguments_before_any_device_work(lib):
    from opensurgsim_gb300 import _lib

    for phases, timeout_ns in ((0, 1_000_000), (1_000_001, 1_000_000), (1, 999), (1, 2_000_000_001)):
        assert lib.gbfem_barrier_selftest(phases, 1, timeout_ns, None, None) == _lib.GBFEM_INVALID_ARG
        assert "barrier_selftest" in _lib.last_error(None)


def test_cpp_facade_compiles_and_links(lib, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ unavailable")
    src = tmp_path / "f.cpp"
    src.write_text('#include "surgsim_compat/surgsim_gb300.h"\n'
                   "int main() { surgsim_gb300::Physics::Fem3DRepresentation r(\"t\");\n"
                   "r.setFemElementType(\"SurgSim::Physics::Fem3DElementCorotationalTetrahedron\");\n"
                   "r.setFemElementType(\"SurgSim::Physics::Fem3DElementTetrahedron\");\n"
                   "r.setFemElementType(\"SurgSim::Physics::Fem3DElementCube\");\n"
                   "surgsim_gb300::Math::LinearSparseSolveAndInverseCG cg; cg.setTolerance(1e-10);\n"
                   "try { r.setFemElementType(\"SurgSim::Physics::Fem1DElementBeam\"); return 1; }\n"
                   "catch (const surgsim_gb300::Framework::AssertionFailure&) {}\n"
                   "const double f[3] = {1, 0, 0};\n"
                   "try { r.addExternalGeneralizedForce(0, std::vector<double>(8, 0.125), f); return 2; }\n"
                   "catch (const surgsim_gb300::Framework::AssertionFailure&) {} return 0; }\n")
    exe = tmp_path / "f"
    subprocess.run([gxx, "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                    "-L" + os.path.join(ROOT, "opensurgsim_gb300"), "-lgbfem", "-o", str(exe)], check=True)
    res = subprocess.run([str(exe)], env=dict(os.environ, LD_LIBRARY_PATH=os.path.join(ROOT, "opensurgsim_gb300")))
    assert res.returncode == 0
