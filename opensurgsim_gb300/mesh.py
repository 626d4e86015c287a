"""Synthetic tetrahedral meshes and the benchmark scene descriptions.

A cube grid of a x b x c cubes of edge h is split into 5 tetrahedra per cube. Node ids follow
OpenSurgSim's ``DivisibleCubeRepresentation`` numbering (``DivisibleCubeRepresentation.cpp:69-72``):
``id = (i*(b+1) + j)*(c+1) + k`` with ``i`` (x) the slowest axis and ``k`` (z) the fastest.

The 5-tet split of a cube is the one used by ``RenderTestFem3DCorotational.cpp:65-72``:
``{4,7,1,2},{4,1,7,5},{4,2,1,0},{4,7,2,6},{1,2,7,3}`` with cube corner ``q = dx + 2*dy + 4*dz``.
Cubes with odd ``i+j+k`` use the x-mirrored split (corner ``q ^ 1``) with two vertices swapped to
keep a positive orientation, so every face diagonal joins the two globally odd-parity corners of
its face and neighbouring cubes share conforming faces.

Scenes are stated in config axes: z is "up", gravity is (0, 0, -9.81) and the bottom face is
z = 0. The step itself takes the gravity vector as a parameter, so no axis permutation is needed.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

_SPLIT_EVEN = np.array([[4, 7, 1, 2], [4, 1, 7, 5], [4, 2, 1, 0], [4, 7, 2, 6], [1, 2, 7, 3]], dtype=np.int64)
_SPLIT_ODD = (_SPLIT_EVEN ^ 1)[:, [0, 1, 3, 2]]  # mirrored in x, orientation restored


@dataclasses.dataclass
class TetMesh:
    """A tetrahedral mesh with per-element material and boundary-condition dofs."""

    nodes: np.ndarray          # (N, 3) float64 rest positions
    tets: np.ndarray           # (E, 4) int32 node ids
    young: np.ndarray          # (E,) float64
    poisson: np.ndarray        # (E,) float64
    density: np.ndarray        # (E,) float64
    bc_dofs: np.ndarray        # (B,) int32 dof ids (3*node + axis)
    dims: tuple = ()
    h: float = 0.0

    @property
    def num_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def num_tets(self) -> int:
        return int(self.tets.shape[0])

    @property
    def num_dofs(self) -> int:
        return 3 * self.num_nodes


def node_id(i, j, k, b, c):
    return (i * (b + 1) + j) * (c + 1) + k


def cube_grid(a: int, b: int, c: int, h: float = 0.01, jitter: float = 0.1, seed: int = 0) -> tuple:
    """Nodes (N,3) and tets (E,4) of an a x b x c cube grid split into 5 tets per cube.

    Interior nodes are jittered uniformly in [-jitter*h, +jitter*h] per axis (PCG64 seeded).
    """
    ii, jj, kk = np.meshgrid(np.arange(a + 1), np.arange(b + 1), np.arange(c + 1), indexing="ij")
    nodes = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64) * h
    if jitter > 0:
        rng = np.random.Generator(np.random.PCG64(seed))
        interior = ((ii > 0) & (ii < a) & (jj > 0) & (jj < b) & (kk > 0) & (kk < c)).ravel()
        noise = rng.uniform(-jitter * h, jitter * h, size=(nodes.shape[0], 3))
        nodes[interior] += noise[interior]
    ci, cj, ck = np.meshgrid(np.arange(a), np.arange(b), np.arange(c), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    corners = np.empty((ci.size, 8), dtype=np.int64)
    for q in range(8):
        dx, dy, dz = q & 1, (q >> 1) & 1, (q >> 2) & 1
        corners[:, q] = node_id(ci + dx, cj + dy, ck + dz, b, c)
    odd = ((ci + cj + ck) & 1).astype(bool)
    tets = np.empty((ci.size, 5, 4), dtype=np.int64)
    tets[~odd] = corners[~odd][:, _SPLIT_EVEN]
    tets[odd] = corners[odd][:, _SPLIT_ODD]
    return nodes, tets.reshape(-1, 4).astype(np.int32)


# Corner order of one hexahedron (Fem3DElementCube node ids) as DivisibleCubeRepresentation.cpp:134-146
# builds it: grid offsets (di, dj, dk) = 000, 100, 110, 010, 001, 101, 111, 011 -- one face cycled,
# then the opposite face cycled the same way, which gives a positive volume.
HEX_CORNERS = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))


def hex_grid(a: int, b: int, c: int, h: float = 0.01, jitter: float = 0.0, seed: int = 0) -> tuple:
    """Nodes (N,3) and hexahedra (E,8) of an a x b x c grid of cubes of edge h (one Fem3DElementCube
    per cube, corners in HEX_CORNERS order). Interior nodes are jittered as in ``cube_grid``."""
    nodes, _ = cube_grid(a, b, c, h=h, jitter=jitter, seed=seed) if jitter > 0 else (None, None)
    if nodes is None:
        ii, jj, kk = np.meshgrid(np.arange(a + 1), np.arange(b + 1), np.arange(c + 1), indexing="ij")
        nodes = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64) * h
    ci, cj, ck = np.meshgrid(np.arange(a), np.arange(b), np.arange(c), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    hexes = np.empty((ci.size, 8), dtype=np.int64)
    for q, (dx, dy, dz) in enumerate(HEX_CORNERS):
        hexes[:, q] = node_id(ci + dx, cj + dy, ck + dz, b, c)
    return nodes, hexes.astype(np.int32)


def scene_hex_cube(a=10, b=10, c=10, h=0.01, seed=0, jitter=0.0, young=1e5, poisson=0.45, density=1000.0,
                   **kw) -> Scene:
    """Hexahedral cube-grid scene with uniform material and the z = 0 face fixed."""
    nodes, hexes = hex_grid(a, b, c, h=h, jitter=jitter, seed=seed)
    E = hexes.shape[0]
    mesh = TetMesh(nodes, hexes, np.full(E, young), np.full(E, poisson), np.full(E, density),
                   face_dofs(a, b, c, 2, 0), (a, b, c), h)
    return Scene(mesh=mesh, name=f"hex{a}x{b}x{c}", element_type=2, **kw)


def scene_divisible_cube(nodes_per_axis: int, **kw) -> Scene:
    """OpenSurgSim's performance-test cube (DivisibleCubeRepresentation.cpp:30-157 with
    Fem3DPerformanceTest.cpp:187-205): nodes_per_axis^3 nodes spanning [-n, n]^3 (n = nodes per axis),
    one hexahedron per grid cell, rho = 980, nu = 0.499, E = 15.3e3, nodes 0, 1 and 2 fixed. Gravity and
    damping keep the representation defaults (gravity (0, -9.81, 0), no Rayleigh damping)."""
    n = int(nodes_per_axis)
    if n < 2:
        raise ValueError("a divisible cube needs at least 2 nodes per axis")
    cells = n - 1
    nodes, hexes = hex_grid(cells, cells, cells, h=2.0 * n / cells)
    nodes -= float(n)
    E = hexes.shape[0]
    mesh = TetMesh(nodes, hexes, np.full(E, 15.3e3), np.full(E, 0.499), np.full(E, 980.0),
                   np.arange(9, dtype=np.int32), (cells, cells, cells), 2.0 * n / cells)
    kw.setdefault("rayleigh_mass", 0.0)
    kw.setdefault("rayleigh_stiffness", 0.0)
    kw.setdefault("gravity", (0.0, -9.81, 0.0))
    kw.setdefault("cg_tolerance", 1e-3)
    kw.setdefault("cg_max_iterations", max(1, int(0.1 * 3 * n ** 3)))
    kw.setdefault("steps", 10)
    return Scene(mesh=mesh, name=f"divisiblecube{n}", element_type=2, **kw)


def signed_volumes(nodes: np.ndarray, tets: np.ndarray) -> np.ndarray:
    p = nodes[tets]
    ab, ac, ad = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    return np.einsum("ij,ij->i", np.cross(ab, ac), ad) / 6.0


def face_dofs(a, b, c, axis: int, index: int) -> np.ndarray:
    """All 3 dofs of every node on the grid face where coordinate `axis` has grid index `index`."""
    ii, jj, kk = np.meshgrid(np.arange(a + 1), np.arange(b + 1), np.arange(c + 1), indexing="ij")
    sel = (ii, jj, kk)[axis] == index
    nid = node_id(ii[sel], jj[sel], kk[sel], b, c).ravel()
    nid.sort()
    return (3 * nid[:, None] + np.arange(3)[None, :]).ravel().astype(np.int32)


@dataclasses.dataclass
class Scene:
    """One mesh plus the step parameters of a benchmark configuration."""

    mesh: TetMesh
    dt: float = 1e-3
    steps: int = 100
    rayleigh_mass: float = 0.01
    rayleigh_stiffness: float = 0.001
    gravity: tuple = (0.0, 0.0, -9.81)
    cg_tolerance: float = 1e-10
    cg_max_iterations: int = 0      # 0: the Eigen default, 2n
    driven_dofs: np.ndarray | None = None   # dofs whose velocity is prescribed before each step
    driven_velocity: float = 0.0            # z velocity of the driven dofs during the ramp
    ramp_steps: int = 0
    name: str = ""
    element_type: int = 0                   # 0 corotational tetrahedra, 1 linear tetrahedra, 2 hexahedra

    def driven_values(self, step: int) -> np.ndarray:
        """Prescribed velocities (per driven dof) before `step`: the z component carries the ramp."""
        vals = np.zeros(self.driven_dofs.size)
        if step < self.ramp_steps:
            vals[2::3] = self.driven_velocity
        return vals


def scene_cube(a=10, b=10, c=10, h=0.01, seed=0, young=1e5, poisson=0.45, density=1000.0, **kw) -> Scene:
    """Single cube-grid scene with uniform material and the z = 0 face fixed (the 10x10x10 case)."""
    nodes, tets = cube_grid(a, b, c, h=h, seed=seed)
    E = tets.shape[0]
    mesh = TetMesh(nodes, tets, np.full(E, young), np.full(E, poisson), np.full(E, density),
                   face_dofs(a, b, c, 2, 0), (a, b, c), h)
    return Scene(mesh=mesh, name=f"cube{a}x{b}x{c}", **kw)


def scene_bar_compression(a=40, b=40, c=160, h=0.004, seed=1, steps=200, dt=1e-3, ramp_steps=50,
                          cg_max_iterations=0) -> Scene:
    """Large bar: per-tet E log-uniform in [1e4, 1e6] Pa, nu uniform in [0.40, 0.49]; z = 0 clamped;
    the z = c*h face is driven at -0.2*L/(ramp_steps*dt) along z for `ramp_steps` steps (a 20%
    axial compression ramp), then held.

    The driven face moves 0.2*c/ramp_steps = 0.64 cube edges per step whatever h is, while an
    elastic wave crosses sqrt(E/rho)*dt/h edges per step. With h = 1 cm the top layers invert within
    three steps and the system stops being positive definite (CG never converges). With h = 4 mm
    (a 16 x 16 x 64 cm bar) no element inverts during the 50 ramp steps (about 450 CG iterations
    per step at tolerance 1e-10); a few elements invert after the ramp, while the bar is held."""
    nodes, tets = cube_grid(a, b, c, h=h, seed=seed)
    E = tets.shape[0]
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    young = np.exp(rng.uniform(math.log(1e4), math.log(1e6), size=E))
    poisson = rng.uniform(0.40, 0.49, size=E)
    clamp = face_dofs(a, b, c, 2, 0)
    top = face_dofs(a, b, c, 2, c)
    mesh = TetMesh(nodes, tets, young, poisson, np.full(E, 1000.0), np.concatenate([clamp, top]), (a, b, c), h)
    L = c * h
    return Scene(mesh=mesh, dt=dt, steps=steps, driven_dofs=top, driven_velocity=-0.2 * L / (ramp_steps * dt),
                 ramp_steps=ramp_steps, name=f"bar{a}x{b}x{c}", cg_max_iterations=cg_max_iterations)


def batch_dims(count: int, lo: float, hi: float, seed: int) -> list:
    """Cube-grid dims with node counts log-uniform in [lo, hi]: a = b = max(1, round(T^(1/3)) - 1),
    c = max(1, round(T/(a+1)^2) - 1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        T = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        a = max(1, int(round(T ** (1.0 / 3.0))) - 1)
        c = max(1, int(round(T / (a + 1) ** 2)) - 1)
        out.append((a, a, c))
    return out


def scenes_batch(count=256, lo=500, hi=50000, seed=3, h=0.01, steps=100) -> list:
    """Independent uneven meshes: per-mesh E log-uniform in [1e4, 1e6], nu = 0.45, z = 0 fixed."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    scenes = []
    for m, (a, b, c) in enumerate(batch_dims(count, lo, hi, seed)):
        E = math.exp(rng.uniform(math.log(1e4), math.log(1e6)))
        s = scene_cube(a, b, c, h=h, seed=seed * 100003 + m, young=E, poisson=0.45, steps=steps)
        s.name = f"batch{m}"
        scenes.append(s)
    return scenes
