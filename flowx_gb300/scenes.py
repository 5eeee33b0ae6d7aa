"""Seeded synthetic scenes for the PBF substep workloads.

No public dataset exists for this path: every workload is a jittered fluid
lattice whose shapes, sizes and parameters are stated here, generated from a
fixed ``numpy.random.default_rng(seed)``.

Conventions shared by all scenes (z up, gravity -9.81 on z as in
``shaders/sph_predict.glsl:37``): particles sit on a lattice of spacing h/2 at
``lo + (i + 0.5) * spacing``, ids run x-fastest, each coordinate is jittered
uniformly in +-0.01 h, initial velocity is zero unless stated, mass is
``1000 * spacing^3`` (the reference's ``rest_density * spacing**3``,
``solver/sph.py:284``) and the rest density is the poly6 density of an
interior lattice particle (``config.lattice_rest_density``).

Workloads:
  dam_break  1 m cube, h 0.1, 20x20x8 = 3,200 particles, seed 0, no collider,
             cohesion 0.1, XSPH 0.01, 4 substeps/frame at 24 fps, 64^3 splat.
  pool       2 m cube, h 0.05, 80x80x48 = 307,200 particles, seed 1; static
             vertical cylinder (r 0.15 m, domain centre) plus a half-height wall
             box 0.1 m thick spanning half the width, voxelised centre-inside
             on a 40^3 uint8 grid (voxel = h); 128^3 splat.
  large      2 m cube, h 0.02, 200x200x100 = 4,000,000 particles, seed 2; a
             0.3 m sphere in free fall from 1.8 m (rests on the floor once it
             lands), re-voxelised every frame on a 100^3 grid; 256^3 splat.
  batched    64 scenes from seed 3 (see ``batched_scenes``).
  inverse    1 m cube, h 0.04, 50x25x16 = 20,000 particles in a block 32% of
             the domain height, seed 4; initial velocity from a 3x3x3 control
             grid of 3-vectors, trilinear (see ``control_velocity``).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .config import (
    SolverConfig,
    SurfaceConfig,
    cell_geometry,
    lattice_rest_density,
    stable_pbf_parameters,
    surface_for_dims,
)

FPS = 24
SUBSTEPS_PER_FRAME = 4
FRAME_DT = 1.0 / FPS


@dataclass
class Primitive:
    """An analytic collider shape, voxelised centre-inside.

    kind 0 = sphere (a = centre, r = radius), 1 = axis-aligned box (a = min,
    b = max), 2 = vertical cylinder (a = base centre, r = radius, b[2] = top z).
    """

    kind: int
    a: tuple
    b: tuple = (0.0, 0.0, 0.0)
    r: float = 0.0


@dataclass
class Scene:
    name: str
    config: SolverConfig
    positions: np.ndarray  # (N, 4) float32, w = 1
    velocities: np.ndarray  # (N, 4) float32, w = 0
    dt: float
    substeps_per_frame: int
    frames: int
    surface: SurfaceConfig
    collider_dims: tuple | None = None
    collider_voxel: float = 0.0
    primitives: list = field(default_factory=list)
    animated: bool = False

    @property
    def n(self) -> int:
        return int(self.positions.shape[0])

    def primitives_at(self, frame: int):
        """Collider primitives at a frame (the large scene's falling sphere)."""
        if not self.animated:
            return list(self.primitives)
        t = frame * FRAME_DT
        out = []
        for p in self.primitives:
            if p.kind == 0:
                z0 = p.a[2]
                z = max(p.r, z0 - 0.5 * 9.81 * t * t)
                out.append(Primitive(0, (p.a[0], p.a[1], z), p.b, p.r))
            else:
                out.append(p)
        return out

    def collider_grid(self, frame: int = 0):
        if self.collider_dims is None:
            return None
        return voxelize(self.primitives_at(frame), self.config.lo, self.collider_voxel, self.collider_dims)


def voxelize(primitives, origin, voxel, dims) -> np.ndarray:
    """uint8 occupancy (z, y, x) of analytic primitives, centre-inside, float64.

    Same layout as the reference's collider grid: origin at the domain's low
    corner, x fastest (collision/__init__.py:245-254, :276-290).
    """
    nx, ny, nz = (int(d) for d in dims)
    xs = origin[0] + (np.arange(nx) + 0.5) * voxel
    ys = origin[1] + (np.arange(ny) + 0.5) * voxel
    zs = origin[2] + (np.arange(nz) + 0.5) * voxel
    z, y, x = np.meshgrid(zs, ys, xs, indexing="ij")
    occ = np.zeros((nz, ny, nx), dtype=bool)
    for p in primitives:
        if p.kind == 0:
            occ |= (x - p.a[0]) ** 2 + (y - p.a[1]) ** 2 + (z - p.a[2]) ** 2 <= p.r * p.r
        elif p.kind == 1:
            occ |= (
                (x >= p.a[0]) & (x <= p.b[0]) & (y >= p.a[1]) & (y <= p.b[1]) & (z >= p.a[2]) & (z <= p.b[2])
            )
        elif p.kind == 2:
            occ |= ((x - p.a[0]) ** 2 + (y - p.a[1]) ** 2 <= p.r * p.r) & (z >= p.a[2]) & (z <= p.b[2])
    return occ.astype(np.uint8)


def sphere_mesh(radius, rings=48, segments=96):
    """A closed UV-sphere triangle mesh about the origin (local space), the
    kind of collider object the reference voxelises: (vertices V x 3 float32,
    triangles T x 3 int32)."""
    verts = [(0.0, 0.0, radius)]
    for i in range(1, rings):
        th = np.pi * i / rings
        for j in range(segments):
            ph = 2.0 * np.pi * j / segments
            verts.append((radius * np.sin(th) * np.cos(ph), radius * np.sin(th) * np.sin(ph), radius * np.cos(th)))
    verts.append((0.0, 0.0, -radius))
    south = len(verts) - 1
    tris = [(0, 1 + j, 1 + (j + 1) % segments) for j in range(segments)]
    for i in range(rings - 2):
        a0, b0 = 1 + i * segments, 1 + (i + 1) * segments
        for j in range(segments):
            jn = (j + 1) % segments
            tris += [(a0 + j, b0 + j, b0 + jn), (a0 + j, b0 + jn, a0 + jn)]
    last = 1 + (rings - 2) * segments
    tris += [(last + j, south, last + (j + 1) % segments) for j in range(segments)]
    return np.asarray(verts, np.float32), np.asarray(tris, np.int32)


def translation(x, y, z):
    """A row-major 4 x 4 world matrix moving local space by (x, y, z)."""
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = (x, y, z)
    return m


def lattice(lo, spacing, counts, h, seed, offset=(0.0, 0.0, 0.0)):
    """Jittered lattice, ids x-fastest. Returns (N, 4) float32 positions, w = 1."""
    nx, ny, nz = counts
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pts = np.asarray(lo, dtype=np.float64) + np.asarray(offset) + (base + 0.5) * spacing
    rng = np.random.default_rng(seed)
    pts += rng.uniform(-0.01 * h, 0.01 * h, size=pts.shape)
    out = np.ones((pts.shape[0], 4), dtype=np.float32)
    out[:, :3] = pts.astype(np.float32)
    return out


def make_config(lo, hi, h, *, cell_rule="h", sigma=0.1, xsph=0.01, epsilon=None, scorr=None, iterations=4,
                reference_defaults=False):
    """Scene parameters.

    cell_rule "h" uses cells of exactly h (the neighbour search's minimum);
    "reference" applies solver/sph.py:286-301 with its MAX_CELLS /
    MAX_CELLS_PER_AXIS budgets. Relaxation and s_corr default to
    ``config.stable_pbf_parameters``; ``reference_defaults`` selects the
    reference's own defaults (relaxation 100, s_corr 0.1,
    domain/__init__.py:85-119), under which the fluid flies apart.
    """
    spacing = h * 0.5
    mass = 1000.0 * spacing**3
    rest = lattice_rest_density(spacing, h, mass)
    if reference_defaults:
        eps_d, k_d = 100.0, 0.1
    else:
        eps_d, k_d = stable_pbf_parameters(spacing, h, mass, rest)
    epsilon = eps_d if epsilon is None else epsilon
    scorr = k_d if scorr is None else scorr
    size = [b - a for a, b in zip(lo, hi)]
    if cell_rule == "h":
        cell = h
        dims = tuple(max(1, math.ceil(axis / cell - 1e-9)) for axis in size)
    elif cell_rule == "reference":
        cell, dims = cell_geometry(lo, hi, max(h, max(size) / 128))
    else:
        raise ValueError(f"unknown cell rule {cell_rule!r}")
    return SolverConfig(
        lo=tuple(float(v) for v in lo),
        hi=tuple(float(v) for v in hi),
        smoothing_radius=float(h),
        spacing=spacing,
        mass=mass,
        rest_density=rest,
        cell_size=float(cell),
        cell_dims=tuple(int(d) for d in dims),
        relaxation=epsilon,
        scorr_strength=scorr,
        surface_tension=sigma,
        viscosity=xsph,
        iterations=iterations,
    )


def _finish(name, config, pos, splat_dims, frames, vel=None, **kw):
    config.particle_count = int(pos.shape[0])
    if vel is None:
        vel = np.zeros_like(pos)
        vel[:, 3] = 0.0
    return Scene(
        name=name,
        config=config,
        positions=pos,
        velocities=vel.astype(np.float32),
        dt=FRAME_DT / SUBSTEPS_PER_FRAME,
        substeps_per_frame=SUBSTEPS_PER_FRAME,
        frames=frames,
        surface=surface_for_dims(config, splat_dims),
        **kw,
    )


def dam_break(cell_rule="h", reference_defaults=False) -> Scene:
    lo, hi, h = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.1
    cfg = make_config(lo, hi, h, cell_rule=cell_rule, reference_defaults=reference_defaults)
    pos = lattice(lo, cfg.spacing, (20, 20, 8), h, seed=0)
    return _finish("dam_break", cfg, pos, 64, 48)


def pool(cell_rule="h", counts=(80, 80, 48), extent=2.0) -> Scene:
    lo, hi, h = (0.0, 0.0, 0.0), (extent, extent, extent), 0.05 * extent / 2.0
    cfg = make_config(lo, hi, h, cell_rule=cell_rule)
    pos = lattice(lo, cfg.spacing, counts, h, seed=1)
    c = extent / 2
    prims = [
        Primitive(2, (c, c, 0.0), (0.0, 0.0, extent), 0.15 * extent / 2),
        Primitive(1, (0.45 * extent / 2, 0.0, 0.0), (0.55 * extent / 2, c, c)),
    ]
    dims = tuple(int(round(extent / h)) for _ in range(3))
    return _finish("pool", cfg, pos, 128, 120, collider_dims=dims, collider_voxel=h, primitives=prims)


def large(cell_rule="h", counts=(200, 200, 100)) -> Scene:
    lo, hi, h = (0.0, 0.0, 0.0), (2.0, 2.0, 2.0), 0.02
    cfg = make_config(lo, hi, h, cell_rule=cell_rule)
    pos = lattice(lo, cfg.spacing, counts, h, seed=2)
    prims = [Primitive(0, (1.0, 1.0, 1.8), (0.0, 0.0, 0.0), 0.3)]
    return _finish(
        "large", cfg, pos, 256, 240, collider_dims=(100, 100, 100), collider_voxel=h, primitives=prims, animated=True
    )


def inverse_problem(n_block=(50, 25, 16), seed=4) -> Scene:
    lo, hi, h = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.04
    cfg = make_config(lo, hi, h)
    pos = lattice(lo, cfg.spacing, n_block, h, seed=seed)
    return _finish("inverse", cfg, pos, 64, 1)


def control_velocity(control: np.ndarray, positions: np.ndarray, lo, hi) -> np.ndarray:
    """Trilinear interpolation of a (3, 3, 3, 3) control grid [node z, y, x, component]
    spanning the domain to per-particle velocities (N, 4) float32."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    u = (positions[:, :3].astype(np.float64) - lo) / (hi - lo) * 2.0
    u = np.clip(u, 0.0, 2.0 - 1e-9)
    i0 = np.floor(u).astype(np.int64)
    f = u - i0
    out = np.zeros((positions.shape[0], 3))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (
                    (f[:, 0] if dx else 1 - f[:, 0])
                    * (f[:, 1] if dy else 1 - f[:, 1])
                    * (f[:, 2] if dz else 1 - f[:, 2])
                )
                out += w[:, None] * control[i0[:, 2] + dz, i0[:, 1] + dy, i0[:, 0] + dx]
    vel = np.zeros((positions.shape[0], 4), dtype=np.float32)
    vel[:, :3] = out
    return vel


def batched_scenes(count=64, seed=3, n_range=(2000, 200000)):
    """The batched workload: ``count`` independent scenes.

    Per scene: particle count log-uniform in n_range, box sides U[0.5, 2] m,
    fill fraction U[0.2, 0.7], h such that the h/2 lattice filling that
    fraction of the box yields the count, 0-2 random axis-aligned box
    colliders voxelised at voxel = h. Cells are exactly h.
    """
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(count):
        target = math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))
        sides = rng.uniform(0.5, 2.0, size=3)
        fill = rng.uniform(0.2, 0.7)
        spacing = (sides[0] * sides[1] * sides[2] * fill / target) ** (1.0 / 3.0)
        h = 2.0 * spacing
        counts = (
            max(1, int(sides[0] / spacing)),
            max(1, int(sides[1] / spacing)),
            max(1, int(sides[2] * fill / spacing)),
        )
        lo = (0.0, 0.0, 0.0)
        hi = tuple(float(v) for v in sides)
        cfg = make_config(lo, hi, h)
        pos = lattice(lo, spacing, counts, h, seed=int(rng.integers(1 << 31)))
        n_col = int(rng.integers(0, 3))
        prims = []
        for _ in range(n_col):
            a = [rng.uniform(0, sides[d] * 0.7) for d in range(3)]
            ext = [rng.uniform(0.1, 0.3) * sides[d] for d in range(3)]
            prims.append(Primitive(1, tuple(a), tuple(a[d] + ext[d] for d in range(3))))
        dims = tuple(max(1, int(math.ceil(side / h - 1e-9))) for side in sides)
        scene = _finish(
            f"batch{s:02d}",
            cfg,
            pos,
            32,
            1,
            collider_dims=dims if prims else None,
            collider_voxel=h if prims else 0.0,
            primitives=prims,
        )
        scenes.append(scene)
    return scenes
