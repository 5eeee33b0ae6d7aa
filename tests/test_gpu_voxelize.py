"""GPU mesh voxeliser (flowx_voxelize_meshes) against its CPU restatement
(oracle/voxelize.py, itself checked against analytic shapes and against the
reference's own voxeliser code): identical occupancy grids for boxes, rotated
and scaled meshes, a lattice-aligned octahedron, a UV sphere, a torus and
unions, up to a 100^3 grid; and against the reference's grids directly; bad
triangle indices are rejected before anything runs."""

import numpy as np
import pytest

import mesh_shapes as S
import test_voxelize_reference as R
from oracle import voxelize as V

pytestmark = pytest.mark.gpu


def _solver(voxels):
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    return Solver(sc.config, sc.positions, sc.velocities, max_collider_voxels=voxels)


def _gpu_grid(s, meshes, dims, voxel, origin):
    s.voxelize_meshes(meshes, dims, voxel, origin)
    return s.collider_occupancy()


CASES = {
    "box": ([(*S.box((-0.43, -0.37, -0.21), (0.52, 0.33, 0.44)), S.identity())], (24, 20, 16), 0.1,
            (-1.0, -0.8, -0.6)),
    "rotated_box": ([(*S.box((-0.3, -0.25, -0.2), (0.35, 0.2, 0.25)),
                      S.rotation((1.0, 2.0, 0.5), 0.7, (0.1, -0.05, 0.08), 1.3))], (24, 20, 16), 0.1,
                    (-1.0, -0.8, -0.6)),
    "octahedron": ([(*S.octahedron((0.15, 0.15, 0.15), 0.5), S.identity())], (24, 20, 16), 0.1,
                   (-1.0, -0.8, -0.6)),
    "torus_union": ([(*S.torus((0.0, 0.0, 0.0), 0.6, 0.22, 64, 32), S.rotation((1.0, 0.0, 0.0), 0.4,
                                                                              (0.1, 0.15, 0.1))),
                     (*S.box((-0.9, -0.7, -0.5), (-0.2, 0.1, 0.3)), S.identity())], (24, 20, 16), 0.1,
                    (-1.0, -0.8, -0.6)),
    "clipped": ([(*S.uv_sphere((0.9, -0.7, 0.55), 0.5, 24, 48), S.rotation((0.3, 1.0, 0.2), 1.1,
                                                                           (0.05, 0.0, 0.0), 1.2))],
                (24, 20, 16), 0.1, (-1.0, -0.8, -0.6)),
    "open_sheet": ([(np.array([[-0.7, -0.5, 0.1], [0.8, -0.4, 0.3], [0.1, 0.9, -0.2]], np.float32),
                     np.array([[0, 1, 2]], np.int32), S.identity())], (24, 20, 16), 0.1, (-1.0, -0.8, -0.6)),
    "sphere_100": ([(*S.uv_sphere((1.0, 1.0, 1.1), 0.3, 48, 96), S.rotation((0.0, 1.0, 1.0), 0.3,
                                                                             (0.05, -0.02, 0.0)))],
                   (100, 100, 100), 0.02, (0.0, 0.0, 0.0)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_equals_oracle(name):
    meshes, dims, voxel, origin = CASES[name]
    want = V.voxelize_meshes(meshes, dims, voxel, origin)
    assert want.any()  # an open sheet marks the centres below it (an odd count above them)
    with _solver(int(np.prod(dims))) as s:
        got = _gpu_grid(s, meshes, dims, voxel, origin)
        again = _gpu_grid(s, meshes, dims, voxel, origin)  # scratch reused
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(again, want)


@pytest.mark.parametrize("name", sorted(R.CASES))
def test_gpu_matches_reference_voxeliser(name):
    """Against the grids of the reference's own voxeliser code
    (tests/test_voxelize_reference.py): equal voxel for voxel, except the
    listed centres that lie exactly on the lattice octahedron's faces."""
    meshes, dims, voxel, origin, _ = R.CASES[name]
    with _solver(int(np.prod(dims))) as s:
        got = _gpu_grid(s, meshes, dims, voxel, origin)
    R.check_against_reference(name, got)


def test_bad_triangle_index_is_rejected():
    from flowx_gb300._lib import FlowxError

    v, t = S.box((0.1, 0.1, 0.1), (0.5, 0.5, 0.5))
    t = t.copy()
    t[3, 1] = 8
    with _solver(10**3) as s:
        with pytest.raises(FlowxError):
            s.voxelize_meshes([(v, t, S.identity())], (10, 10, 10), 0.1, (0.0, 0.0, 0.0))


def test_mesh_collider_drives_the_substep():
    """A mesh box and the analytic box of the same extent give the same grid,
    so the same substep (EXACT arithmetic)."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    lo, hi = (0.52, 0.03, 0.03), (0.78, 0.97, 0.47)
    dims, voxel = (10, 10, 10), 0.1
    out = []
    for use_mesh in (False, True):
        with Solver(sc.config, sc.positions, sc.velocities, max_collider_voxels=1000, exact=True) as s:
            if use_mesh:
                s.voxelize_meshes([(*S.box(lo, hi), S.identity())], dims, voxel)
            else:
                s.voxelize([scenes.Primitive(1, lo, hi, 0.0)], dims, voxel)
            s._build_grid(0.0)
            for _ in range(4):
                s._substep(sc.dt)
            out.append(s.read("positions"))
    np.testing.assert_array_equal(out[0], out[1])
