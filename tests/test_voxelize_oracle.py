"""The mesh voxeliser's CPU restatement (oracle/voxelize.py) against analytic
shapes: occupancy by the parity of crossings of the vertical ray above each
voxel centre, as collision/__init__.py:304-367 defines it. Closed meshes of
boxes (axis-aligned and rotated), an octahedron whose vertices and edges lie
exactly on voxel columns (the watertight edge rule), a UV sphere and a torus
(a surface of genus one), unions, singular and out-of-grid meshes."""

import numpy as np

import mesh_shapes as S
from oracle import voxelize as V

DIMS = (24, 20, 16)
VOXEL = 0.1
ORIGIN = (-1.0, -0.8, -0.6)


def _grid(meshes, dims=DIMS, voxel=VOXEL, origin=ORIGIN):
    return V.voxelize_meshes(meshes, dims, voxel, origin).astype(bool)


def test_axis_aligned_box_matches_the_box_exactly():
    lo, hi = (-0.43, -0.37, -0.21), (0.52, 0.33, 0.44)
    g = _grid([(*S.box(lo, hi), S.identity())])
    x, y, z = S.centres(DIMS, VOXEL, ORIGIN)
    want = (x > lo[0]) & (x < hi[0]) & (y > lo[1]) & (y < hi[1]) & (z > lo[2]) & (z < hi[2])
    assert want.sum() > 100
    np.testing.assert_array_equal(g, want)


def test_rotated_scaled_box_matches_its_half_spaces():
    lo, hi = (-0.3, -0.25, -0.2), (0.35, 0.2, 0.25)
    m = S.rotation((1.0, 2.0, 0.5), 0.7, translate=(0.1, -0.05, 0.08), scale=1.3)
    g = _grid([(*S.box(lo, hi), m)])
    x, y, z = S.centres(DIMS, VOXEL, ORIGIN)
    md = m.astype(np.float64)
    inv = np.linalg.inv(md[:3, :3])
    p = np.stack([x - md[0, 3], y - md[1, 3], z - md[2, 3]], -1) @ inv.T
    margin = np.minimum.reduce([p[..., 0] - lo[0], hi[0] - p[..., 0], p[..., 1] - lo[1], hi[1] - p[..., 1],
                                p[..., 2] - lo[2], hi[2] - p[..., 2]])
    sure = np.abs(margin) > 1e-6
    assert (margin > 0).sum() > 100
    np.testing.assert_array_equal(g[sure], (margin > 0)[sure])


def test_octahedron_on_the_lattice_is_watertight():
    # centre on a voxel centre, vertices on voxel centres: columns pass exactly
    # through vertices and edges, and many centres lie exactly on faces
    c = (-1.0 + 11.5 * VOXEL, -0.8 + 9.5 * VOXEL, -0.6 + 7.5 * VOXEL)
    r = 5 * VOXEL
    v, t = S.octahedron(c, r)
    g = _grid([(v, t, S.identity())])
    x, y, z = S.centres(DIMS, VOXEL, ORIGIN)
    d = np.abs(x - np.float32(c[0])) + np.abs(y - np.float32(c[1])) + np.abs(z - np.float32(c[2]))
    strict_in, strict_out = d < r - 1e-6, d > r + 1e-6
    assert strict_in.sum() > 100
    assert g[strict_in].all() and not g[strict_out].any()


def test_sphere_and_torus_agree_away_from_the_surface():
    c = (0.15, 0.2, 0.18)
    g = _grid([(*S.uv_sphere(c, 0.55, 32, 64), S.identity())])
    x, y, z = S.centres(DIMS, VOXEL, ORIGIN)
    d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
    sure = np.abs(d - 0.55) > 0.55 * 0.01
    np.testing.assert_array_equal(g[sure], (d < 0.55)[sure])

    m = S.rotation((1.0, 0.0, 0.0), 0.4, translate=(0.1, 0.15, 0.1))
    g = _grid([(*S.torus((0.0, 0.0, 0.0), 0.6, 0.22, 64, 32), m)])
    md = m.astype(np.float64)
    p = np.stack([x - md[0, 3], y - md[1, 3], z - md[2, 3]], -1) @ np.linalg.inv(md[:3, :3]).T
    q = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - 0.6
    dist = np.sqrt(q**2 + p[..., 2] ** 2) - 0.22
    sure = np.abs(dist) > 0.22 * 0.03
    assert (dist < 0)[sure].sum() > 100
    np.testing.assert_array_equal(g[sure], (dist < 0)[sure])


def test_union_singular_and_outside():
    a = (*S.box((-0.9, -0.7, -0.5), (-0.2, 0.1, 0.3)), S.identity())
    b = (*S.octahedron((0.3, 0.2, 0.1), 0.45), S.identity())
    ga, gb = _grid([a]), _grid([b])
    assert ga.any() and gb.any()
    np.testing.assert_array_equal(_grid([a, b]), ga | gb)
    flat = S.identity()
    flat[2, 2] = 0.0  # an axis scaled to zero: the reference voxelises nothing
    assert not _grid([(*S.box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)), flat)]).any()
    assert not _grid([(*S.box((5.0, 5.0, 5.0), (6.0, 6.0, 6.0)), S.identity())]).any()
    assert not _grid([(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32), S.identity())]).any()


def test_index_range_is_the_reference_rule():
    v, _ = S.box((-0.43, -0.37, -0.21), (0.52, 0.33, 0.44))
    lo, hi = V.index_range(v, S.identity(), DIMS, VOXEL, ORIGIN)
    o = [float(np.float32(x)) for x in ORIGIN]
    vox = float(np.float32(VOXEL))
    f = [float(np.float32(x)) for x in (-0.43, -0.37, -0.21)]
    g = [float(np.float32(x)) for x in (0.52, 0.33, 0.44)]
    import math

    assert lo == [max(0, math.floor((f[r] - o[r]) / vox)) for r in range(3)]
    assert hi == [min(DIMS[r], math.ceil((g[r] - o[r]) / vox)) for r in range(3)]


def test_scene_sphere_mesh_is_closed_and_voxelises_as_the_sphere():
    """flowx_gb300.scenes.sphere_mesh (the bench's collider mesh): every edge
    shared by exactly two triangles, and its voxels those of the analytic
    sphere away from the surface."""
    from flowx_gb300 import scenes

    v, t = scenes.sphere_mesh(0.3, 24, 48)
    e = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert (counts == 2).all()
    c = (0.05, -0.1, 0.12)
    g = _grid([(v, t, scenes.translation(*c))])
    x, y, z = S.centres(DIMS, VOXEL, ORIGIN)
    d = np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2)
    sure = np.abs(d - 0.3) > 0.3 * 0.02
    assert (d < 0.3)[sure].sum() > 50
    np.testing.assert_array_equal(g[sure], (d < 0.3)[sure])
