"""Solver configuration, push-constant packing and seeding for the PBF substep.

Host-side restatement of the parts of Flow-X's ``solver/sph.py`` and
``solver/surface.py`` that decide *what* the GPU passes compute:

* ``SolverConfig`` / ``resolve_config``   - ``solver/sph.py:195-303``
* ``SolverConfig.substep_dt``              - ``solver/sph.py:228-249``
* ``seed_counts`` / ``seed_positions_reference`` - ``solver/sph.py:306-347``
* ``push_constant_values`` / ``pack_push`` - ``solver/sph.py:433-461`` and the
  128-byte block of ``shaders/sph_common.glsl:10-17``
* ``SurfaceConfig`` / ``resolve_surface`` / ``splat_push_values`` -
  ``solver/surface.py:92-140`` and ``:201-233``
* ``collider_grid_geometry``              - ``collision/__init__.py:245-254``

The reference hard-codes its particle, cell and splat-sample budgets
(``MAX_PARTICLES``, ``MAX_CELLS``, ``MAX_CELLS_PER_AXIS``, ``MAX_SAMPLES``).
Here they are keyword parameters whose defaults are the reference's values,
so large scenes (4M particles, 1e6 cells, 256^3 splat grids) can lift them.
"""

from __future__ import annotations

import math
import random
import struct
from dataclasses import dataclass, field

import numpy as np

# solver/sph.py:82-111
LOCAL_GROUP_SIZE = 64
GRAVITY = -9.81
BOUNDARY_DAMPING = 0.35
MAX_PARTICLES = 16384
MAX_CELLS = 262144
MAX_CELLS_PER_AXIS = 128
CFL_FACTOR = 0.25
# solver/gpu_util.py:28-30
TEXTURE_WIDTH = 256
# shaders/sph_common.glsl:27-30
MAX_CELL_SCAN = 512
# solver/surface.py:45-53
MAX_SAMPLES = 1 << 20
SURFACE_CELL_RADIUS = 2

PUSH_FIELDS = (
    ("i", "i_layout"),
    ("i", "i_grid"),
    ("i", "i_sort"),
    ("f", "f_lo"),
    ("f", "f_hi"),
    ("f", "f_sph"),
    ("f", "f_sim"),
    ("i", "i_collider"),
)


def float_bits(value: float) -> int:
    """floatBitsToInt of a float32, as solver/sph.py:440-441 packs scorr/sigma."""
    return struct.unpack("<i", struct.pack("<f", float(value)))[0]


def bits_float(bits: int) -> float:
    return struct.unpack("<f", struct.pack("<i", int(bits)))[0]


@dataclass
class SolverConfig:
    """Resolved parameters of one scene (solver/sph.py:195-226)."""

    lo: tuple
    hi: tuple
    smoothing_radius: float
    spacing: float
    mass: float
    rest_density: float
    cell_size: float
    cell_dims: tuple
    particle_count: int = 0
    fill_fraction: float = 0.0
    relaxation: float = 100.0
    scorr_strength: float = 0.1
    surface_tension: float = 0.0
    viscosity: float = 0.1
    max_substeps: int = 24
    iterations: int = 4
    gravity: float = GRAVITY
    damping: float = BOUNDARY_DAMPING
    extra: dict = field(default_factory=dict)

    @property
    def particle_radius(self) -> float:
        return self.spacing * 0.5

    @property
    def cell_count(self) -> int:
        return int(self.cell_dims[0]) * int(self.cell_dims[1]) * int(self.cell_dims[2])

    @property
    def sorted_count(self) -> int:
        """Bitonic sort width, the next power of two >= particle_count
        (solver/sph.py:353). Kept for the reference key-buffer layout."""
        return max(2, 1 << (max(1, self.particle_count) - 1).bit_length())

    def substep_dt(self, frame_dt: float):
        """(substeps, dt) for one frame, solver/sph.py:228-249."""
        gravity_dt = CFL_FACTOR * math.sqrt(self.smoothing_radius / abs(GRAVITY))
        kinematic = self.viscosity / max(self.rest_density, 1e-6)
        viscous_dt = 0.125 * self.smoothing_radius**2 / max(kinematic, 1e-12)
        limit = min(gravity_dt, viscous_dt)
        steps = min(max(1, math.ceil(frame_dt / limit)), self.max_substeps)
        return steps, min(frame_dt / steps, limit)


def seed_counts(size, fill_height, spacing):
    """Particles per axis for a lattice inset by half a spacing (solver/sph.py:306-313)."""
    margin = spacing
    return (
        max(1, int((size[0] - margin) / spacing)),
        max(1, int((size[1] - margin) / spacing)),
        max(1, int(max(fill_height - margin, 0.0) / spacing)),
    )


def cell_geometry(lo, hi, cell_size, max_cells=MAX_CELLS, max_cells_per_axis=MAX_CELLS_PER_AXIS):
    """Cell size and dims under the reference rule (solver/sph.py:286-301).

    ``cell_size`` is the starting size (the reference passes
    ``max(h, longest / MAX_CELLS_PER_AXIS)``); it grows by 1.5x, at most 8
    times, while the grid exceeds ``max_cells``.
    """
    size = [float(b) - float(a) for a, b in zip(lo, hi)]
    dims = None
    for _ in range(8):
        dims = tuple(
            min(max_cells_per_axis, max(1, math.ceil(axis / cell_size))) for axis in size
        )
        if dims[0] * dims[1] * dims[2] <= max_cells:
            break
        cell_size *= 1.5
    return cell_size, dims


def resolve_config(
    lo,
    hi,
    *,
    fluid_level=50.0,
    smoothing_radius=0.1,
    rest_density=1000.0,
    relaxation=100.0,
    iterations=4,
    scorr_strength=0.1,
    surface_tension=0.0,
    viscosity=0.1,
    max_substeps=24,
    max_particles=MAX_PARTICLES,
    max_cells=MAX_CELLS,
    max_cells_per_axis=MAX_CELLS_PER_AXIS,
) -> SolverConfig:
    """The reference's _resolve_config (solver/sph.py:252-303), budgets as parameters."""
    size = [float(b) - float(a) for a, b in zip(lo, hi)]
    h = float(smoothing_radius)
    spacing = h * 0.5
    fill_height = size[2] * fluid_level / 100.0
    for _ in range(8):
        nx, ny, nz = seed_counts(size, fill_height, spacing)
        if nx * ny * nz <= max_particles:
            break
        spacing *= (nx * ny * nz / max_particles) ** (1 / 3)
        h = spacing * 2.0
    mass = rest_density * spacing**3
    cell_size, dims = cell_geometry(
        lo, hi, max(h, max(size) / max_cells_per_axis), max_cells, max_cells_per_axis
    )
    return SolverConfig(
        lo=tuple(float(v) for v in lo),
        hi=tuple(float(v) for v in hi),
        smoothing_radius=h,
        spacing=spacing,
        mass=mass,
        rest_density=float(rest_density),
        cell_size=cell_size,
        cell_dims=dims,
        fill_fraction=fluid_level / 100.0,
        relaxation=float(relaxation),
        scorr_strength=float(scorr_strength),
        surface_tension=float(surface_tension),
        viscosity=float(viscosity),
        max_substeps=int(max_substeps),
        iterations=int(iterations),
    )


def seed_positions_reference(config: SolverConfig, max_particles=MAX_PARTICLES, dtype=np.float32) -> np.ndarray:
    """The reference's jittered seed lattice (solver/sph.py:316-347).

    Uses Python's ``random.Random(0)`` exactly as the reference does, so the
    same domain seeds the same particles. Returns (N, 4) ``dtype``, w = 1
    (float64 keeps the reference's Python floats exactly).
    """
    size = [b - a for a, b in zip(config.lo, config.hi)]
    nx, ny, nz = seed_counts(size, size[2] * config.fill_fraction, config.spacing)
    rng = random.Random(0)
    jitter = config.spacing * 0.1
    base = [v + config.spacing * 0.5 for v in config.lo]
    values = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                if len(values) >= max_particles:
                    return np.asarray(values, dtype=dtype)
                values.append(
                    (
                        base[0] + i * config.spacing + rng.uniform(-jitter, jitter),
                        base[1] + j * config.spacing + rng.uniform(-jitter, jitter),
                        base[2] + k * config.spacing + rng.uniform(-jitter, jitter),
                        1.0,
                    )
                )
    return np.asarray(values, dtype=dtype)


def push_constant_values(config: SolverConfig, dt, i_collider=(1, 1, 1, 0), sort_k=0, sort_j=0):
    """The shared push-constant block as {name: 4-tuple} (solver/sph.py:433-461).

    ``i_collider`` is (dims.xyz, floatBitsToInt(voxel)); voxel 0 means no
    collider (solver/sph.py:420-430).
    """
    return {
        "i_layout": (config.particle_count, TEXTURE_WIDTH, TEXTURE_WIDTH, config.sorted_count),
        "i_grid": (*config.cell_dims, config.cell_count),
        "i_sort": (sort_k, sort_j, float_bits(config.scorr_strength), float_bits(config.surface_tension)),
        "f_lo": (*config.lo, config.cell_size),
        "f_hi": (*config.hi, config.particle_radius),
        "f_sph": (config.smoothing_radius, config.mass, config.rest_density, config.relaxation),
        "f_sim": (config.viscosity, dt, config.gravity, config.damping),
        "i_collider": tuple(i_collider),
    }


def pack_push(values: dict) -> bytes:
    """Serialise a push dict into the 128-byte block (int32/float32 little-endian)."""
    out = b""
    for kind, name in PUSH_FIELDS:
        slot = name if name in values else ("i_surface" if name == "i_sort" else name)
        vec = values[slot]
        out += struct.pack("<4i" if kind == "i" else "<4f", *vec)
    assert len(out) == 128
    return out


def collider_binding(dims=None, voxel_size=0.0):
    """i_collider for a grid (solver/sph.py:413-430): (1,1,1,0) means none."""
    if dims is None or voxel_size <= 0.0:
        return (1, 1, 1, 0)
    return (int(dims[0]), int(dims[1]), int(dims[2]), float_bits(voxel_size))


def collider_grid_geometry(lo, hi, resolution):
    """(origin, voxel_size, dims) of the collider grid (collision/__init__.py:245-254)."""
    size = [b - a for a, b in zip(lo, hi)]
    longest = max(size)
    if longest <= 0.0:
        return tuple(lo), 0.0, (0, 0, 0)
    voxel = longest / resolution
    dims = tuple(max(1, round(axis / voxel)) for axis in size)
    return tuple(lo), voxel, dims


@dataclass
class SurfaceConfig:
    """Splat-grid geometry (solver/surface.py:92-95)."""

    dims: tuple
    spacing: float
    kernel_radius: float
    lo: tuple
    iso: float = 0.5

    @property
    def sample_count(self) -> int:
        return int(self.dims[0]) * int(self.dims[1]) * int(self.dims[2])


def _kernel_radius(config: SolverConfig, spacing):
    # solver/surface.py:115-122
    return min(max(config.smoothing_radius, spacing * 1.5), SURFACE_CELL_RADIUS * config.cell_size)


def resolve_surface(config: SolverConfig, resolution=48, iso=0.5, max_samples=MAX_SAMPLES):
    """The reference's surface.resolve (solver/surface.py:97-140), budget as a parameter."""
    size = [b - a for a, b in zip(config.lo, config.hi)]
    spacing = max(max(size) / max(resolution, 1), 1e-6)
    dims = None
    for _ in range(8):
        margin = _kernel_radius(config, spacing)
        extent = [axis + 2 * margin for axis in size]
        dims = tuple(max(2, int(-(-axis // spacing)) + 1) for axis in extent)
        if dims[0] * dims[1] * dims[2] <= max_samples:
            break
        spacing *= 1.25
    radius = _kernel_radius(config, spacing)
    lo = tuple(v - radius for v in config.lo)
    return SurfaceConfig(dims=dims, spacing=spacing, kernel_radius=radius, lo=lo, iso=iso)


def surface_for_dims(config: SolverConfig, samples_per_axis: int, iso=0.5) -> SurfaceConfig:
    """A splat grid with exactly ``samples_per_axis`` lattice points along the
    longest axis, laid out by the reference's rule (grid starts one kernel
    radius below the domain and spans one past it, solver/surface.py:123-139).
    """
    size = [b - a for a, b in zip(config.lo, config.hi)]
    longest = max(size)
    spacing = longest / max(samples_per_axis - 1, 1)
    for _ in range(50):
        margin = _kernel_radius(config, spacing)
        new_spacing = (longest + 2 * margin) / (samples_per_axis - 1)
        if abs(new_spacing - spacing) < 1e-15:
            break
        spacing = new_spacing
    radius = _kernel_radius(config, spacing)
    dims = tuple(
        max(2, min(samples_per_axis, int(math.ceil((axis + 2 * radius) / spacing - 1e-9)) + 1))
        for axis in size
    )
    lo = tuple(v - radius for v in config.lo)
    return SurfaceConfig(dims=dims, spacing=spacing, kernel_radius=radius, lo=lo, iso=iso)


def splat_push_values(config: SolverConfig, surface: SurfaceConfig, dt, i_collider):
    """The splat pass's block: the SPH block with i_sort -> i_surface, f_sph.x ->
    kernel radius and f_hi -> (surface lo, 0) (solver/surface.py:212-233)."""
    values = push_constant_values(config, dt, i_collider)
    values.pop("i_sort")
    values["i_surface"] = (*surface.dims, float_bits(surface.spacing))
    values["f_sph"] = (surface.kernel_radius, *values["f_sph"][1:])
    values["f_hi"] = (*surface.lo, 0.0)
    return values


def lattice_rest_density(spacing: float, h: float, mass: float) -> float:
    """Poly6 density (self included) of an interior particle of a perfect cubic
    lattice, in float64: the "rest density from the poly6 kernel at seeding"
    used by the synthetic scenes. Same kernel as shaders/sph_common.glsl:68-91.
    """
    reach = int(math.ceil(h / spacing))
    coef = 315.0 / (64.0 * math.pi * h**9)
    total = 0.0
    for i in range(-reach, reach + 1):
        for j in range(-reach, reach + 1):
            for k in range(-reach, reach + 1):
                r2 = (i * i + j * j + k * k) * spacing * spacing
                if r2 < h * h:
                    total += coef * (h * h - r2) ** 3
    return mass * total


def lattice_constraint_denominator(spacing: float, h: float, mass: float, rest_density: float) -> float:
    """(|sum grad|^2 + sum |grad|^2) / rho0^2 of sph_lambda.glsl:60-73 for an
    interior particle of a perfect cubic lattice, in float64 (the first term is
    zero by symmetry)."""
    reach = int(math.ceil(h / spacing))
    coef = -45.0 / (math.pi * h**6)
    total = 0.0
    for i in range(-reach, reach + 1):
        for j in range(-reach, reach + 1):
            for k in range(-reach, reach + 1):
                r2 = (i * i + j * j + k * k) * spacing * spacing
                if 1e-12 < r2 < h * h:
                    r = math.sqrt(r2)
                    g = mass * coef * (h - r) ** 2
                    total += g * g
    return total / (rest_density * rest_density)


def mass_consistent_relaxation(spacing: float, h: float, mass: float, rest_density: float, floor=100.0) -> float:
    """Relaxation epsilon under which the reference's position update equals the
    mass-consistent Jacobi PBF step at the seeded lattice.

    sph_delta.glsl:78-84 divides by rho0 without the particle mass that its
    lambda denominator (sph_lambda.glsl:64, :73) carries, so every correction is
    1/m times the mass-consistent one. With lambda = -C / (D + eps), choosing
    eps = D * (1/m - 1) makes (1/rho0) * lambda equal (m/rho0) * (-C / D).
    """
    d = lattice_constraint_denominator(spacing, h, mass, rest_density)
    return max(floor, d * (1.0 / mass - 1.0))


def scorr_for_displacement(h: float, rest_density: float, displacement: float) -> float:
    """s_corr strength k at which one neighbour at distance h/2 contributes a
    correction of ``displacement`` (metres) through sph_delta.glsl:72-78:
    k * (W(h/2) / W(0.2 h))^4 * |grad W_spiky(h/2)| / rho0 = displacement."""
    coef = 315.0 / (64.0 * math.pi * h**9)
    h2 = h * h
    w_q = coef * (h2 - (0.2 * h) ** 2) ** 3
    w = coef * (h2 - (0.5 * h) ** 2) ** 3
    grad = 45.0 / (math.pi * h**6) * (0.5 * h) ** 2
    return displacement * rest_density / ((w / w_q) ** 4 * grad)


def stable_pbf_parameters(spacing: float, h: float, mass: float, rest_density: float,
                          relaxation_factor: float = 31.0, scorr_displacement: float = 1e-4):
    """(relaxation, scorr_k) for the synthetic workloads.

    The reference's update lacks the particle mass in sph_delta.glsl:84, so at
    mass < 1 kg its Jacobi step over-shoots by 1/m and the fluid flies apart
    within a substep at its own defaults (relaxation 100, s_corr 0.1). The
    workloads instead use the relaxation that makes that update equal the
    mass-consistent step with a relaxation of ``relaxation_factor`` times the
    lattice denominator D, i.e. eps = D * ((1 + f) / m - 1), and an s_corr
    strength whose per-neighbour correction at h/2 is
    ``scorr_displacement * h``. With f = 31 the free-surface particles, whose
    density constraint the reference does not clamp, stay within a cell of the
    grid they were sorted into; at f = 7 a few escape it in deep columns,
    lose their own density term (it drops to the 1e-6 floor) and XSPH then
    drives their neighbours to ~1e6 m/s.
    """
    d = lattice_constraint_denominator(spacing, h, mass, rest_density)
    eps = d * ((1.0 + relaxation_factor) / mass - 1.0)
    k = scorr_for_displacement(h, rest_density, scorr_displacement * h)
    return eps, k


def config_from_push(values: dict) -> SolverConfig:
    """A SolverConfig whose push_constant_values() reproduces ``values``
    (float32 fields round-trip exactly)."""
    f_lo, f_hi, f_sph, f_sim = (tuple(float(v) for v in values[k]) for k in ("f_lo", "f_hi", "f_sph", "f_sim"))
    i_grid, i_sort = values["i_grid"], values["i_sort"]
    cfg = SolverConfig(
        lo=f_lo[:3],
        hi=f_hi[:3],
        smoothing_radius=f_sph[0],
        spacing=2.0 * f_hi[3],
        mass=f_sph[1],
        rest_density=f_sph[2],
        cell_size=f_lo[3],
        cell_dims=tuple(int(v) for v in i_grid[:3]),
        particle_count=int(values["i_layout"][0]),
        relaxation=f_sph[3],
        scorr_strength=bits_float(i_sort[2]),
        surface_tension=bits_float(i_sort[3]),
        viscosity=f_sim[0],
        gravity=f_sim[2],
        damping=f_sim[3],
    )
    return cfg
