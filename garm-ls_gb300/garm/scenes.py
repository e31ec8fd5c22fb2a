"""Seeded synthetic scenes for the per-step pipeline.

A scene is an "n^D MAC grid on [0,1]^D, dx = 1/n, solid walls", i.e.
StaggeredGrid(boundaryWidth=2, spacing=1/n, resolution=n+4, center=0.5)
(Source/Core/StaggeredGrid.h:27-36), with φ built from implicit surfaces
combined by `min` as LevelSetLiquid::unionLevelSet does
(Source/Core/LevelSetLiquid.cpp:700-707).  Signed distances follow
ImplicitBox / ImplicitSphere / ImplicitPlane (Source/Core/ImplicitSurface.h:7-126),
evaluated in FP64 in the same operation order, so every form of the pipeline
starts from bit-identical inputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .capi import GridDesc, field_shapes, grid_desc


@dataclass
class Scene:
    name: str
    grid: GridDesc
    phi: np.ndarray             # cell field, numpy shape reversed(resolution)
    velocity: np.ndarray        # concatenated face arrays (.sav layout)
    meta: dict = field(default_factory=dict)

    @property
    def interior_cells(self) -> int:
        n = 1
        for a in range(self.grid.dim):
            n *= self.grid.resolution[a] - 2 * self.grid.boundary_width
        return n


def unit_grid(dim: int, n: int, bw: int = 2) -> GridDesc:
    return grid_desc(dim, [n + 2 * bw] * dim, 1.0 / n, [0.5] * dim, bw)


def _origin(grid: GridDesc) -> list[float]:
    return [grid.center[a] - float(grid.resolution[a]) * grid.spacing / 2 for a in range(grid.dim)]


def cell_positions(grid: GridDesc) -> list[np.ndarray]:
    """Per-axis cell-centre coordinates broadcastable to the cell array (Grid::position)."""
    dim, dx = grid.dim, grid.spacing
    o = _origin(grid)
    out = []
    for a in range(dim):
        co = o[a] + 1.0 * dx / 2
        x = co + np.arange(grid.resolution[a], dtype=np.float64) * dx
        shape = [1] * dim
        shape[dim - 1 - a] = grid.resolution[a]
        out.append(x.reshape(shape))
    return out


def box_sdf(pos: list[np.ndarray], min_corner, lengths) -> np.ndarray:
    """ImplicitBox::signedDistance (ImplicitSurface.h:51-56)."""
    dim = len(pos)
    c = [min_corner[a] + lengths[a] / 2 for a in range(dim)]
    h = [lengths[a] / 2 for a in range(dim)]
    phi = [np.abs(pos[a] - c[a]) - h[a] for a in range(dim)]
    phi = np.broadcast_arrays(*phi)
    inside = np.ones(phi[0].shape, dtype=bool)
    for p in phi:
        inside &= p <= 0
    mx = phi[0].copy()
    for p in phi[1:]:
        mx = np.maximum(mx, p)
    s = np.zeros(phi[0].shape)
    for p in phi:
        q = np.maximum(p, 0.0)
        s = s + q * q
    return np.where(inside, mx, np.sqrt(s))


def sphere_sdf(pos: list[np.ndarray], center, radius: float) -> np.ndarray:
    """ImplicitSphere::signedDistance (ImplicitSurface.h:22): |p - c| - r."""
    s = 0.0
    for a in range(len(pos)):
        d = pos[a] - center[a]
        s = s + d * d
    return np.sqrt(s) - radius


def plane_sdf(pos: list[np.ndarray], point, normal) -> np.ndarray:
    """ImplicitPlane::signedDistance (ImplicitSurface.h:123): (p - x0)·n̂."""
    nn = np.sqrt(sum(v * v for v in normal))
    n = [v / nn for v in normal]
    s = 0.0
    for a in range(len(pos)):
        s = s + (pos[a] - point[a]) * n[a]
    return s


def zero_velocity(grid: GridDesc) -> np.ndarray:
    shapes = field_shapes(grid)
    return np.zeros(sum(int(np.prod(s)) for s in shapes["faces"]), dtype=np.float64)


def velocity_with(grid: GridDesc, axis: int, value: float) -> np.ndarray:
    shapes = field_shapes(grid)
    parts = [np.full(int(np.prod(s)), value if a == axis else 0.0) for a, s in enumerate(shapes["faces"])]
    return np.concatenate(parts)


def dam_break(dim: int, n: int, extent=None) -> Scene:
    """Liquid column {x < 0.4, y < 0.6} (2D) or {x < 0.4, y < 0.5, z < 0.6} (3D), at rest.

    The column is the box [-1, e]^D, so inside the unit domain its signed
    distance is that of the half-open region — the walls do not add a surface.
    """
    if extent is None:
        extent = (0.4, 0.6) if dim == 2 else (0.4, 0.5, 0.6)
    grid = unit_grid(dim, n)
    pos = cell_positions(grid)
    lo = [-1.0] * dim
    phi = box_sdf(pos, lo, [extent[a] - lo[a] for a in range(dim)])
    phi = np.minimum(np.full(phi.shape, np.inf), phi)
    return Scene(f"dam_break_{dim}d_{n}", grid, np.ascontiguousarray(phi), zero_velocity(grid), {"extent": list(extent)})


def drop(n: int, seed: int = 0, dim: int = 3, radius: float = 0.12, depth: float = 0.3, speed: float = -1.0) -> Scene:
    """Pool of depth 0.3 plus a sphere of radius 0.12 at a seeded centre in
    [0.3,0.7]^2 x [0.6,0.8] (y up), all faces at u_y = -1."""
    rng = np.random.default_rng(seed)
    grid = unit_grid(dim, n)
    pos = cell_positions(grid)
    if dim == 3:
        c = [rng.uniform(0.3, 0.7), rng.uniform(0.6, 0.8), rng.uniform(0.3, 0.7)]
        pn = [0.0, 1.0, 0.0]
        p0 = [0.0, depth, 0.0]
    else:
        c = [rng.uniform(0.3, 0.7), rng.uniform(0.6, 0.8)]
        pn = [0.0, 1.0]
        p0 = [0.0, depth]
    phi = np.full(np.broadcast_shapes(*[p.shape for p in pos]), np.inf)
    phi = np.minimum(phi, plane_sdf(pos, p0, pn))
    phi = np.minimum(phi, sphere_sdf(pos, c, radius))
    return Scene(f"drop_{dim}d_{n}_s{seed}", grid, np.ascontiguousarray(phi), velocity_with(grid, 1, speed),
                 {"center": c, "radius": radius, "depth": depth})


def random_pool_scene(n: int, seed: int, dim: int = 3) -> Scene:
    """1-3 seed-placed spheres of radius 0.05-0.15 over a pool of depth 0.1-0.4."""
    rng = np.random.default_rng(seed)
    grid = unit_grid(dim, n)
    pos = cell_positions(grid)
    depth = rng.uniform(0.1, 0.4)
    pn = [0.0] * dim; pn[1] = 1.0
    p0 = [0.0] * dim; p0[1] = depth
    phi = np.full(np.broadcast_shapes(*[p.shape for p in pos]), np.inf)
    phi = np.minimum(phi, plane_sdf(pos, p0, pn))
    spheres = []
    for _ in range(int(rng.integers(1, 4))):
        r = rng.uniform(0.05, 0.15)
        c = [rng.uniform(0.2, 0.8) for _ in range(dim)]
        c[1] = rng.uniform(depth + r + 0.05, 0.85)
        phi = np.minimum(phi, sphere_sdf(pos, c, r))
        spheres.append((c, r))
    return Scene(f"pool_{dim}d_{n}_s{seed}", grid, np.ascontiguousarray(phi), zero_velocity(grid),
                 {"depth": depth, "spheres": spheres})


def frame_time_steps(max_speed_fn, n_steps: int, frame_rate: int = 25, cfl: float = 1.0, dx: float = 1.0):
    """Simulator::advanceTimeBySteps dt policy (Common/Util/Simulator.cpp:102-128):
    dt = cfl*dx/max|u| clamped to the frame end and halved when two steps remain.
    Yields n_steps values of dt; `max_speed_fn()` is called before each step."""
    target = 1.0 / frame_rate
    time = 0.0
    done_steps = 0
    while done_steps < n_steps:
        m = max_speed_fn()
        dt = cfl * dx / m if m > 0 else float("inf")
        if time + dt >= target:
            dt = target - time
            time = 0.0
        elif time + 2 * dt >= target:
            dt = (target - time) / 2
            time += dt
        else:
            time += dt
        done_steps += 1
        yield dt
