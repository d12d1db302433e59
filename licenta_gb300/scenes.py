"""Seeded synthetic inputs of the five cloth workloads.

The reference builds its cloth with VisualBodyFactory::CreateMeshProps
(Rendering/VisualBodyFactory.cpp:343-391) and pins two corners
(Managers/MastersSimulationManager.cpp:67-77); the triangle topology here is
that generator's, placed as a 1 m x 1 m grid in the XZ plane at y = 1 m with
a seeded uniform jitter on every coordinate.  Parameters the workloads leave
open keep the reference defaults of Managers/MastersSimulationManager.cpp
:33-62.

The grid topology and the default parameters are built here in numpy (the
same values as the library's lc_mesh_grid and lc_default_params, which a CPU
test holds byte for byte), so the workloads can be generated without loading
the CUDA library; only the icosphere calls it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _ffi


@dataclass
class ClothSpec:
    positions: np.ndarray      # (V, 3) float32
    indices: np.ndarray        # (T, 3) uint32
    pinned: np.ndarray         # (V,) uint8
    params: _ffi.ClothParams
    meta: dict = field(default_factory=dict)
    # static triangle collider: (vertices (N, 3) float32, indices (M, 3)
    # uint32, winding "ccw" | "cw" seen from the free side)
    collider: tuple | None = None

    @property
    def num_vertices(self) -> int:
        return int(self.positions.shape[0])

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])


def grid_indices(n: int) -> np.ndarray:
    """VisualBodyFactory::CreateMeshProps (Rendering/VisualBodyFactory.cpp
    :343-391) for an n x n grid: two triangles per quad in row-major quad
    order, the quad's diagonal alternating with the parity of i + j."""
    if n < 2:
        return np.zeros((0, 3), dtype=np.uint32)
    i, j = np.meshgrid(np.arange(n - 1, dtype=np.int64), np.arange(n - 1, dtype=np.int64), indexing="ij")
    a, b = n * i + j, n * (i + 1) + j
    c, d = a + 1, b + 1
    even = ((i + j) % 2 == 0)[..., None]
    t0 = np.where(even, np.stack([a, b, c], -1), np.stack([a, b, d], -1))
    t1 = np.where(even, np.stack([c, b, d], -1), np.stack([d, c, a], -1))
    return np.stack([t0, t1], axis=2).reshape(-1, 3).astype(np.uint32)


def default_params() -> _ffi.ClothParams:
    """The reference's ClothParams defaults (Managers/MastersSimulationManager
    .cpp:33-62, timestep from Core/Utils.hpp:18-19) plus the extension
    defaults of lc_cloth_params: the values lc_default_params fills."""
    f = np.float32
    p = _ffi.ClothParams()
    p.timestep = float(f(f(1000.0) / f(60.0)) / f(1000.0))
    p.kFriction, p.kStretch, p.kShear, p.kBend = 0.1, 0.99, 0.7, 0.1
    p.kDamp, p.kSpringDamp, p.thickness, p.objectMass = 0.05, 0.2, 0.0, 0.525
    p.globalVelDamp, p.strainLimit = 0.01, 0.15
    p.gravity[:] = (0.0, -0.0981, 0.0)
    p.minWindDir[:] = (-0.04, -0.1, -0.1)
    p.startWindDir[:] = (0.02, 0.095, 0.45)
    p.maxWindDir[:] = (0.04, 0.135, 0.4)
    p.windMinVariation, p.windMaxVariation, p.windOn = 0.0, 0.2, 1
    p.worldMin[:] = (0.0, 0.0, 0.0)
    p.worldMax[:] = (1.0, 1.0, 1.0)
    p.dims[:] = (60, 60)
    p.solverIterations, p.ccdIterations, p.BVHChunkSize, p.benchmarkSample = 6, 5, 64, 1000
    p.useTriangleBending = p.colorContacts = p.useFriction = 0
    p.thicknessFromMesh, p.mortonMode, p.refLeafAabbQuirk, p.groundOn = 1, _ffi.LC_MORTON_REF63, 1, 1
    p.mortonOrigin[:] = (0.0, 0.0, 0.0)
    p.mortonScale, p.windSeed, p.sphereOn, p.sphereRadius = 1.0, 0, 0, 0.0
    return p


def icosphere(depth: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Rendering/VisualBodyFactory.cpp:259-341 (unwelded vertices; the faces
    turn clockwise seen from outside)."""
    t = _ffi.lib().lc_mesh_icosphere(depth, None, None)
    v = np.empty((3 * t // 4 * 2, 3), dtype=np.float32)
    idx = np.empty((t, 3), dtype=np.uint32)
    _ffi.lib().lc_mesh_icosphere(depth, v.ctypes.data_as(C.c_void_p), idx.ctypes.data_as(C.c_void_p))
    return v * np.float32(radius) + np.asarray(center, dtype=np.float32), idx


def grid_positions(n: int, rng: np.random.Generator, jitter: float = 1e-4, y: float = 1.0,
                   span: float = 1.0, origin=(0.0, 0.0)) -> np.ndarray:
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    p = np.stack([origin[0] + span * i / (n - 1), np.full(i.shape, y), origin[1] + span * j / (n - 1)], axis=-1)
    p = p.reshape(-1, 3) + rng.uniform(-jitter, jitter, size=(n * n, 3))
    return p.astype(np.float32)


def corner_pins(n: int) -> np.ndarray:
    """The two pinned vertices of Managers/MastersSimulationManager.cpp:67-77."""
    p = np.zeros(n * n, dtype=np.uint8)
    p[0] = 1
    p[(n - 1) * n] = 1
    return p


def base_params(iterations: int, stiffness: float, dt: float = 1.0 / 60.0) -> _ffi.ClothParams:
    p = default_params()
    p.timestep = dt
    p.gravity[:] = (0.0, -9.81, 0.0)
    p.solverIterations = iterations
    p.kStretch = stiffness
    p.kBend = stiffness
    p.windOn = 0
    return p


def set_constant_wind(p: _ffi.ClothParams, wind) -> None:
    """A constant wind: the reference update with zero variation clamped to itself."""
    p.windOn = 1
    p.startWindDir[:] = wind
    p.minWindDir[:] = wind
    p.maxWindDir[:] = wind
    p.windMinVariation = 0.0
    p.windMaxVariation = 0.0


def small_cloth(seed: int = 0, n: int = 32, iterations: int = 10, stiffness: float = 0.9,
                thickness: float = 0.01) -> ClothSpec:
    """32x32 grid, two pinned corners, 10 iterations, stiffness 0.9, 0.01 m thickness."""
    rng = np.random.default_rng(seed)
    p = base_params(iterations, stiffness)
    p.thicknessFromMesh = 0
    p.thickness = thickness
    p.dims[:] = (n, n)
    return ClothSpec(grid_positions(n, rng), grid_indices(n), corner_pins(n), p,
                     dict(workload="plain-small", n=n, steps=120))


def large_cloth(seed: int = 0, n: int = 512, iterations: int = 20, stiffness: float = 0.9,
                sphere_radius: float = 0.3, mesh: bool = False) -> ClothSpec:
    """512x512 grid centred over a sphere of radius 0.3 m at the origin,
    dropped from y = 1 m (no pins), 20 iterations.  The sphere is the
    reference's analytic sphere collider (CudaPBD::SetSpherePos), or with
    mesh=True the icosphere of subdivision 5 (20,480 faces) as a static
    triangle collider instead."""
    rng = np.random.default_rng(seed)
    p = base_params(iterations, stiffness)
    p.dims[:] = (n, n)
    p.worldMin[:] = (-1.0, -1.0, -1.0)
    p.worldMax[:] = (1.0, 1.0, 1.0)
    p.mortonOrigin[:] = (-1.0, -1.0, -1.0)
    p.mortonScale = 0.5
    p.sphereOn = 1
    p.spherePos[:] = (0.0, 0.0, 0.0)
    p.sphereRadius = sphere_radius
    pos = grid_positions(n, rng, origin=(-0.5, -0.5))
    coll = None
    if mesh:
        p.sphereOn = 0
        coll = (*icosphere(5, sphere_radius), "cw")
    return ClothSpec(pos, grid_indices(n), np.zeros(n * n, dtype=np.uint8), p,
                     dict(workload="plain-large", n=n, steps=300, mesh=mesh), collider=coll)


def icosphere_cloth(seed: int = 0, n: int = 32, depth: int = 3, radius: float = 0.3, iterations: int = 10,
                    stiffness: float = 0.9, height: float = 0.5, span: float = 1.0) -> ClothSpec:
    """An n x n cloth `span` metres wide centred over the origin at y =
    `height` (no pins), dropped onto a static icosphere of subdivision
    `depth` and radius `radius` at the origin, given as a triangle collider
    (lc_batch_set_collider); the analytic sphere is off.  World box and
    Morton frame [-1, 1]^3."""
    rng = np.random.default_rng(seed)
    p = base_params(iterations, stiffness)
    p.dims[:] = (n, n)
    p.worldMin[:] = (-1.0, -1.0, -1.0)
    p.worldMax[:] = (1.0, 1.0, 1.0)
    p.mortonOrigin[:] = (-1.0, -1.0, -1.0)
    p.mortonScale = 0.5
    pos = grid_positions(n, rng, y=height, span=span, origin=(-span / 2, -span / 2))
    return ClothSpec(pos, grid_indices(n), np.zeros(n * n, dtype=np.uint8), p,
                     dict(workload="icosphere", n=n, depth=depth, r=radius),
                     collider=(*icosphere(depth, radius), "cw"))


def batched_cloths(seed: int = 0, count: int = 256, n_min: int = 16, n_max: int = 192,
                   iterations: int = 10) -> list[ClothSpec]:
    """256 cloths, side drawn from U{16..192}, stiffness U[0.5, 1.0], constant
    wind U[-2, 2] m/s^2 on x and z, two pinned corners each."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(n_min, n_max + 1, size=count)
    ks = rng.uniform(0.5, 1.0, size=count)
    winds = rng.uniform(-2.0, 2.0, size=(count, 2))
    out = []
    for c in range(count):
        n = int(sides[c])
        p = base_params(iterations, float(ks[c]))
        p.dims[:] = (n, n)
        set_constant_wind(p, (float(winds[c, 0]), 0.0, float(winds[c, 1])))
        out.append(ClothSpec(grid_positions(n, rng), grid_indices(n), corner_pins(n), p,
                             dict(workload="batched", n=n, k=float(ks[c]))))
    return out


def batched_sphere_cloths(seed: int = 0, count: int = 128, n_min: int = 32, n_max: int = 128,
                          iterations: int = 10, mesh: bool = False) -> list[ClothSpec]:
    """The batched differentiable workload: 128 unpinned cloths, side drawn
    from U{32..128}, 1 m square centred over the origin at y = 1 m, each
    dropped onto its own sphere at the origin with radius U[0.2, 0.4] m (the
    reference's analytic sphere collider, CudaPBD::SetSpherePos), stiffness
    0.9, 10 iterations.  mesh=True: each sphere is an icosphere of
    subdivision 4 (5,120 faces) given as a static triangle collider, the
    analytic sphere off."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(n_min, n_max + 1, size=count)
    radii = rng.uniform(0.2, 0.4, size=count)
    out = []
    for c in range(count):
        n = int(sides[c])
        p = base_params(iterations, 0.9)
        p.dims[:] = (n, n)
        p.worldMin[:] = (-1.0, -1.0, -1.0)
        p.worldMax[:] = (1.0, 1.0, 1.0)
        p.mortonOrigin[:] = (-1.0, -1.0, -1.0)
        p.mortonScale = 0.5
        p.sphereOn = 1
        p.spherePos[:] = (0.0, 0.0, 0.0)
        p.sphereRadius = float(radii[c])
        coll = None
        if mesh:
            p.sphereOn = 0
            coll = (*icosphere(4, float(radii[c])), "cw")
        out.append(ClothSpec(grid_positions(n, rng, origin=(-0.5, -0.5)), grid_indices(n),
                             np.zeros(n * n, dtype=np.uint8), p, dict(workload="batched-sphere", n=n,
                                                                      r=float(radii[c]), mesh=mesh),
                             collider=coll))
    return out


def adjoint_cloth(seed: int = 0, n: int = 64, stiffness: float = 0.9, wind=(0.0, 0.0, 0.0)) -> ClothSpec:
    """64x64 grid, 10 iterations (differentiable rollout workload)."""
    rng = np.random.default_rng(seed)
    p = base_params(10, stiffness)
    p.dims[:] = (n, n)
    if any(w != 0.0 for w in wind):
        set_constant_wind(p, tuple(float(w) for w in wind))
    return ClothSpec(grid_positions(n, rng), grid_indices(n), corner_pins(n), p,
                     dict(workload="adjoint", n=n, steps=60))


def equal_code_cloth(seed: int = 26, copies: int = 4, n: int = 10,
                     offset=(0.0009218, 0.0, -0.0031407)) -> ClothSpec:
    """A 10x10 grid 0.1 m wide around the world origin plus `copies`
    near-coincident loose triangles (2e-8 m apart, shifted by `offset`) beside
    its centre.  Their Morton codes are equal, and a run of >= 3 equal codes
    makes two internal nodes of the Karras hierarchy claim one child, so the
    refit never reaches some nodes, the root among them (their boxes stay
    zero, where the reference's would stay stale).  World box and Morton
    frame [-1, 1]^3, 10 iterations, stiffness 0.9."""
    rng = np.random.default_rng(seed)
    p = base_params(10, 0.9)
    p.worldMin[:] = (-1.0, -1.0, -1.0)
    p.worldMax[:] = (1.0, 1.0, 1.0)
    p.mortonOrigin[:] = (-1.0, -1.0, -1.0)
    p.mortonScale = 0.5
    pos = grid_positions(n, rng, y=0.0, span=0.1, origin=(-0.05, -0.05))
    tri = np.array([[0.002, 0.0005, 0.001], [0.004, 0.0005, 0.003], [0.001, 0.0005, 0.004]], np.float32)
    extra = np.concatenate([tri + np.float32(2e-8 * k) for k in range(copies)]).astype(np.float32)
    extra += np.asarray(offset, dtype=np.float32)
    idx = np.concatenate([grid_indices(n), (pos.shape[0] + np.arange(3 * copies, dtype=np.uint32)).reshape(-1, 3)])
    return ClothSpec(np.concatenate([pos, extra]).astype(np.float32), idx.astype(np.uint32),
                     np.zeros(pos.shape[0] + 3 * copies, dtype=np.uint8), p,
                     dict(workload="equal-codes", copies=copies))


def random_triangle_boxes(count: int, seed: int = 0):
    """LBVH microbenchmark input: first vertex uniform in the unit cube, two
    edges of length U[1e-3, 5e-3] in uniformly random directions; returns the
    (min, max) boxes, each (count, 3) float32."""
    rng = np.random.default_rng(seed)
    v0 = rng.uniform(0.0, 1.0, size=(count, 3))
    dirs = rng.normal(size=(count, 2, 3))
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    lens = rng.uniform(1e-3, 5e-3, size=(count, 2, 1))
    v1 = v0 + dirs[:, 0] * lens[:, 0]
    v2 = v0 + dirs[:, 1] * lens[:, 1]
    tri = np.stack([v0, v1, v2], axis=1).astype(np.float32)
    return tri.min(axis=1), tri.max(axis=1)
