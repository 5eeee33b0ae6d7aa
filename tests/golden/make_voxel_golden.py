"""Generate ``tests/golden/voxel_reference.npz``: collider occupancy grids made
by the reference's own voxeliser code (collision/__init__.py: ``_rebuild_grid``
:304-367, ``_point_inside`` :264-274, ``_index_range`` :257-262, the union of
``_rebuild_solver_grid`` :225-242, ``_domain_grid_geometry`` :245-254 and
``world_bounds``, domain/__init__.py:212-218), run outside Blender:

    python tests/golden/make_voxel_golden.py [--ref CHECKOUT]

Blender objects are stand-ins holding a local triangle mesh, its local bound
box and a row-major world matrix; the BVH ray cast is the stand-in of
``reference_host.BVHTree`` (nearest hit, Moller-Trumbore in float64), since
Blender's own BVH is compiled code that is not here. Everything else - the
domain grid geometry, the index range over the transformed bound box, the
ray from each voxel centre taken into local space through the inverse
matrix, the re-launch 1e-4 past every hit, the parity, the singular-matrix
rule, the union - is the reference's code itself.

Stored per case: the meshes (local vertices, triangles, world matrix), the
domain grid (origin, voxel, dims, from the reference's geometry function) and
the reference's union grid ((nz, ny, nx) uint8).
"""

from __future__ import annotations

import argparse
import importlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import mesh_shapes as S  # noqa: E402
import reference_host as RH  # noqa: E402
from oracle import refpath  # noqa: E402


def _corners(lo, hi):
    return [(x, y, z) for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])]


class _Object:
    """The slice of a Blender mesh object the voxeliser reads."""

    def __init__(self, name, vertices, triangles, matrix):
        v = np.asarray(vertices, np.float32).reshape(-1, 3)
        self.name = name
        self.type = "MESH"
        self.matrix_world = RH.Matrix(np.asarray(matrix, np.float32).astype(np.float64))
        lo, hi = v.min(axis=0).astype(np.float64), v.max(axis=0).astype(np.float64)
        self.bound_box = _corners(lo, hi)
        self.data = types.SimpleNamespace(
            vertices=[types.SimpleNamespace(co=tuple(float(c) for c in row)) for row in v],
            polygons=[types.SimpleNamespace(vertices=tuple(int(i) for i in t)) for t in np.asarray(triangles)],
        )

    def evaluated_get(self, _depsgraph):
        return self


class _Domain:
    def __init__(self, lo, hi, resolution):
        self.name = "Domain"
        self.matrix_world = RH.Matrix(np.eye(4))
        self.bound_box = _corners(lo, hi)
        self.flowx_domain = types.SimpleNamespace(resolution=resolution)


DOMAIN = ((-1.0, -0.8, -0.6), (1.4, 1.2, 1.0), 24)


def cases():
    """name -> (meshes [(vertices, triangles, matrix)], domain (lo, hi, resolution))."""
    sphere = S.uv_sphere((0.137, 0.211, 0.163), 0.47)
    return {
        "sphere_rotated": ([(*sphere, S.rotation((0.3, 1.0, 0.2), 0.9, (0.05, -0.02, 0.04)))], DOMAIN),
        "box_rotated_scaled": ([(*S.box((-0.3, -0.25, -0.2), (0.35, 0.2, 0.25)),
                                 S.rotation((1.0, 2.0, 0.5), 0.7, (0.1, -0.05, 0.08), 1.3))], DOMAIN),
        "torus_tilted": ([(*S.torus((0.0, 0.0, 0.0), 0.5, 0.18, 48, 24),
                           S.rotation((1.0, 0.3, 0.0), 1.1, (0.21, 0.17, 0.2)))], DOMAIN),
        "union": ([(*S.uv_sphere((0.0, 0.0, 0.0), 0.27), S.rotation((0.0, 0.0, 1.0), 0.3, (-0.49, -0.41, -0.27))),
                   (*S.box((0.0, 0.0, 0.0), (0.6, 0.5, 0.5)), S.rotation((0.0, 1.0, 0.0), 0.2, (0.31, 0.29, 0.12)))],
                  DOMAIN),
        "singular_and_sphere": ([(*S.box((-0.2, -0.2, -0.2), (0.2, 0.2, 0.2)),
                                  np.diag([1.0, 1.0, 0.0, 1.0]).astype(np.float32)),
                                 (*S.uv_sphere((0.33, 0.27, 0.41), 0.3), S.identity())], DOMAIN),
        "clipped": ([(*S.uv_sphere((0.0, 0.0, 0.0), 0.4), S.rotation((1.0, 1.0, 1.0), 0.5, (1.28, 1.09, 0.87)))],
                    DOMAIN),
        "falling_sphere_100": ([(*S.uv_sphere((0.0, 0.0, 0.0), 0.3, 48, 96),
                                 S.rotation((0.0, 0.0, 1.0), 0.0, (1.0, 1.0, 0.9)))],
                               ((0.0, 0.0, 0.0), (2.0, 2.0, 2.0), 100)),
        "octahedron_on_lattice": ([(*S.octahedron((0.15, 0.15, 0.15), 0.5), S.identity())], DOMAIN),
    }


def reference_grid(collision, meshes, domain):
    lo, hi, res = domain
    dom = _Domain(lo, hi, res)
    origin, voxel, dims = collision._domain_grid_geometry(dom)
    collision._grids.clear()
    collision._mesh_fingerprints.clear()
    collision._solver_grid.update(texture=None, voxel_size=0.0, dims=(1, 1, 1))
    for k, (v, t, m) in enumerate(meshes):
        collision._rebuild_grid(dom, _Object(f"Collider{k}", v, t, m))
    tex = collision._solver_grid["texture"]
    nx, ny, nz = dims
    if tex is None:
        grid = np.zeros((nz, ny, nx), np.uint8)
    else:
        grid = (np.asarray(tex.data.values, np.float32) > 0.5).astype(np.uint8).reshape(nz, ny, nx)
    return grid, (float(origin.x), float(origin.y), float(origin.z)), float(voxel), tuple(int(d) for d in dims)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $FLOWX_REFERENCE)")
    args = ap.parse_args()
    args.ref = args.ref or refpath.checkout()
    RH.load(args.ref)
    collision = importlib.import_module("flowx_reference.collision")
    out, meta = {}, {}
    for name, (meshes, domain) in cases().items():
        grid, origin, voxel, dims = reference_grid(collision, meshes, domain)
        out[f"{name}_grid"] = grid
        for k, (v, t, m) in enumerate(meshes):
            out[f"{name}_mesh{k}_vertices"] = np.asarray(v, np.float32)
            out[f"{name}_mesh{k}_triangles"] = np.asarray(t, np.int32)
            out[f"{name}_mesh{k}_matrix"] = np.asarray(m, np.float32)
        meta[name] = {"meshes": len(meshes), "origin": origin, "voxel": voxel, "dims": dims}
        print(f"{name}: dims {dims}, voxel {voxel:.6g}, {int(grid.sum())} occupied")
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "voxel_reference.npz"), **out)


if __name__ == "__main__":
    main()
