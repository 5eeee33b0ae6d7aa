"""GPU marching cubes against the reference's own extract
(solver/marching_cubes.py:191-280; meshes in tests/golden/mc_golden.npz made
by make_mc_golden.py): same vertices in the same order with bit-identical
float64 coordinates, same triangles. Plus the reference tests' properties:
closed meshes (every edge shared by exactly two triangles), outward windings
(positive signed volume), nothing below the iso value."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("sphere", "noise", "splat", "empty")


def _golden():
    return np.load(os.path.join(HERE, "golden", "mc_golden.npz"))


def _lattice(z, name):
    lat = z[f"{name}_lattice"]
    return tuple(int(v) for v in lat[:3]), tuple(float(v) for v in lat[3:6]), float(lat[6]), float(lat[7])


def _watertight(tris):
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    e.sort(axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    return bool((counts == 2).all())


def _signed_volume(v, t):
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


@pytest.mark.parametrize("name", FIELDS)
def test_extract_matches_reference_bit_exact(name):
    from flowx_gb300.surface import MarchingCubes

    z = _golden()
    dims, origin, spacing, iso = _lattice(z, name)
    mc = MarchingCubes(0)
    verts, tris = mc.extract(z[f"{name}_field"], dims, origin, spacing, iso)
    np.testing.assert_array_equal(tris, z[f"{name}_triangles"])
    np.testing.assert_array_equal(verts, z[f"{name}_vertices"])
    # a second extraction on the same object reuses its buffers
    verts2, tris2 = mc.extract(z[f"{name}_field"], dims, origin, spacing, iso)
    np.testing.assert_array_equal(tris2, tris)
    np.testing.assert_array_equal(verts2, verts)


def test_closed_surfaces_and_outward_windings():
    from flowx_gb300.surface import extract

    z = _golden()
    for name in ("sphere", "noise"):
        dims, origin, spacing, iso = _lattice(z, name)
        verts, tris = extract(z[f"{name}_field"], dims, origin, spacing, iso)
        assert len(tris) > 1000 and _watertight(tris), name
    dims, origin, spacing, iso = _lattice(z, "sphere")
    verts, tris = extract(z["sphere_field"], dims, origin, spacing, iso)
    vol = _signed_volume(verts, tris)
    assert vol > 0.0 and abs(vol - 4.0 / 3.0 * np.pi * 0.6**3) < 0.03 * 4.0 / 3.0 * np.pi * 0.6**3


def test_solver_surface_mesh_matches_reference_on_oracle_splat():
    """Splat and extraction on the device for the dam break after seeding: the
    splat is bit-exact with the oracle's, so the mesh equals the reference's
    mesh of the oracle's splat."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver

    z = _golden()
    sc = scenes.dam_break()
    with Solver(sc.config, sc.positions, sc.velocities, max_surface_samples=sc.surface.sample_count,
                exact=True) as s:
        s._build_grid(0.0)
        verts, tris = s.surface_mesh(sc.surface, sc.dt)
    np.testing.assert_array_equal(tris, z["splat_triangles"])
    np.testing.assert_array_equal(verts, z["splat_vertices"])


def _smooth_field(dims, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = np.zeros((nz, ny, nx), np.float64)
    for _ in range(6):
        k = rng.uniform(0.02, 0.12, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        f += np.sin(k[0] * x + ph[0]) * np.sin(k[1] * y + ph[1]) * np.sin(k[2] * z + ph[2])
    return f.astype(np.float32).reshape(-1)


@pytest.mark.parametrize("dims,iso", [((192, 160, 144), 0.0), ((97, 131, 64), 0.35)])
def test_extract_matches_oracle_beyond_fixtures(dims, iso):
    """Lattices larger and more ragged than the fixtures: the device mesh
    equals the oracle's (oracle/mc.py, itself pinned to the reference's
    meshes), vertices bit-identical."""
    from flowx_gb300.surface import MarchingCubes
    from oracle import mc as oracle_mc

    field = _smooth_field(dims, seed=sum(dims))
    mc = MarchingCubes(0)
    verts, tris = mc.extract(field, dims, (-0.3, 0.1, 0.7), 0.0123, iso)
    ov, ot = oracle_mc.extract(field, dims, (-0.3, 0.1, 0.7), 0.0123, iso)
    assert len(ot) > 10000
    np.testing.assert_array_equal(tris, ot)
    np.testing.assert_array_equal(verts, ov)
    mc.close()


def test_solver_surface_mesh_matches_oracle_pool():
    """The 307,200-particle pool scene after two substeps: the device mesh of
    its 128^3 splat equals the oracle's mesh of the same splat grid."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver
    from oracle import mc as oracle_mc

    sc = scenes.pool()
    with Solver(sc.config, sc.positions, sc.velocities, collider=sc.collider_grid(0),
                collider_voxel=sc.collider_voxel, max_surface_samples=sc.surface.sample_count) as s:
        s._build_grid(0.0)
        for _ in range(2):
            s._substep(sc.dt)
        verts, tris = s.surface_mesh(sc.surface, sc.dt)
        field = s.update_surface(sc.surface, sc.dt)
    ov, ot = oracle_mc.extract(field, sc.surface.dims, sc.surface.lo, sc.surface.spacing, sc.surface.iso)
    assert len(ot) > 10000
    np.testing.assert_array_equal(tris, ot)
    np.testing.assert_array_equal(verts, ov)


def test_destroy_after_the_extraction_stream_is_gone():
    """An extraction on a solver's stream, the solver closed first (its stream
    destroyed), then the marching-cubes object: destroy must not use the
    caller's stream of the last extraction."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver
    from flowx_gb300.surface import MarchingCubes

    sc = scenes.dam_break()
    mc = MarchingCubes(0)
    s = Solver(sc.config, sc.positions, sc.velocities, max_surface_samples=sc.surface.sample_count)
    s._build_grid(0.0)
    verts, tris = s.surface_mesh(sc.surface, sc.dt, mc)
    assert len(tris) > 0
    s.close()
    mc.close()
