"""The mesh voxeliser's CPU restatement (oracle/voxelize.py) against grids made
by the reference's own voxeliser code (collision/__init__.py ``_rebuild_grid``,
``_point_inside``, ``_index_range``, the union of ``_rebuild_solver_grid``;
fixtures by tests/golden/make_voxel_golden.py, where only Blender's BVH ray
cast is a stand-in). Rotated, scaled and translated meshes (the inverse-matrix
path), a union, a singular transform next to a sphere, a mesh clipped by the
domain and the benchmark's falling sphere on 100^3 voxels are equal voxel for
voxel. The one listed exception: an octahedron placed on the lattice, 15 of
whose voxel centres lie exactly on its faces; a point on the surface is
neither inside nor outside, and the two rules decide it differently (the ray
cast from the rounding of its hit distance, the restatement by an exact
comparison)."""

import json
import os

import numpy as np
import pytest

from oracle import voxelize as V

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "voxel_reference.npz")
# the lattice-aligned octahedron of make_voxel_golden.py: centre and radius
OCTA_CENTRE, OCTA_R = np.array([0.15, 0.15, 0.15]), 0.5


def load_cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    out = {}
    for name, m in meta.items():
        meshes = [(z[f"{name}_mesh{k}_vertices"], z[f"{name}_mesh{k}_triangles"], z[f"{name}_mesh{k}_matrix"])
                  for k in range(m["meshes"])]
        out[name] = (meshes, tuple(m["dims"]), m["voxel"], tuple(m["origin"]), z[f"{name}_grid"])
    return out


CASES = load_cases()


def check_against_reference(name, got):
    _, dims, voxel, origin, want = CASES[name]
    assert got.shape == want.shape
    diff = np.argwhere(got != want)
    if name != "octahedron_on_lattice":
        assert len(diff) == 0, f"{name}: {len(diff)} voxels differ from the reference, e.g. {diff[:5].tolist()}"
        return
    assert len(diff) == 15, len(diff)
    for k, j, i in diff:
        c = np.asarray(origin) + (np.array([i, j, k]) + 0.5) * voxel
        assert abs(np.abs(c - OCTA_CENTRE).sum() - OCTA_R) < 1e-12, (i, j, k)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_voxeliser(name):
    meshes, dims, voxel, origin, want = CASES[name]
    assert want.sum() > 0
    check_against_reference(name, V.voxelize_meshes(meshes, dims, voxel, origin))
