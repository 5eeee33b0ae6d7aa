"""CPU restatement of the mesh collider voxeliser (test infrastructure).

Follows collision/__init__.py of Flow-X: ``_rebuild_grid`` (:304-367) marks
a voxel of the domain grid (origin at the domain's low corner, x fastest,
centre ``origin + (i + 0.5) * voxel``) occupied when ``_point_inside``
(:264-274) finds an odd number of hits on the ray from the voxel's centre
along world +z, for the voxels of ``_index_range`` (:257-262) over the
mesh's ``world_bounds`` (domain/__init__.py:212-218: the box of the eight
transformed corners of the local bounds); a singular matrix marks nothing
(:340-353); colliders are unioned (:225-242).

The reference counts hits with Blender's BVH ray casts, re-launched 1e-4
past each hit; neither Blender nor its BVH exists here, so this restatement
counts the crossings exactly: world-space triangles in float64, a crossing
when the column point lies inside the triangle's xy projection (edge
functions evaluated from the lexicographically smaller endpoint, so that two
triangles sharing an edge see exactly opposite values, and points exactly on
an edge or vertex decided as if displaced by (eps, eps^2)), and a centre
counts a crossing strictly above it. It is pinned against the reference's own
voxeliser code run outside Blender, with only the BVH ray cast a stand-in
(tests/golden/make_voxel_golden.py, tests/test_voxelize_reference.py: equal
on every case but voxel centres lying exactly on a mesh face), and against
analytic shapes (tests/test_voxelize_oracle.py); the GPU voxeliser is
checked against it bit for bit.

Only the tests use this module.
"""

from __future__ import annotations

import math

import numpy as np


def world_vertices(vertices, matrix):
    """World-space vertices (float64): M [v; 1], each row summed as
    ((m0 x + m1 y) + m2 z) + m3."""
    v = np.asarray(vertices, np.float32).reshape(-1, 3).astype(np.float64)
    m = np.asarray(matrix, np.float32).reshape(4, 4).astype(np.float64)
    out = np.empty_like(v)
    for r in range(3):
        out[:, r] = ((m[r, 0] * v[:, 0] + m[r, 1] * v[:, 1]) + m[r, 2] * v[:, 2]) + m[r, 3]
    return out


def index_range(vertices, matrix, dims, voxel, origin):
    """[lo, hi) voxel index ranges per axis of the mesh's world bounds."""
    v = np.asarray(vertices, np.float32).reshape(-1, 3).astype(np.float64)
    m = np.asarray(matrix, np.float32).reshape(4, 4).astype(np.float64)
    llo, lhi = v.min(axis=0), v.max(axis=0)
    wlo = np.full(3, np.inf)
    whi = np.full(3, -np.inf)
    for corner in range(8):
        p = (lhi[0] if corner & 1 else llo[0], lhi[1] if corner & 2 else llo[1], lhi[2] if corner & 4 else llo[2])
        for r in range(3):
            w = ((m[r, 0] * p[0] + m[r, 1] * p[1]) + m[r, 2] * p[2]) + m[r, 3]
            wlo[r] = min(wlo[r], w)
            whi[r] = max(whi[r], w)
    vox = float(np.float32(voxel))
    o = [float(np.float32(x)) for x in origin]
    lo = [int(max(0.0, math.floor((wlo[r] - o[r]) / vox))) for r in range(3)]
    hi = [int(min(float(dims[r]), math.ceil((whi[r] - o[r]) / vox))) for r in range(3)]
    return lo, hi


def _edge_fn(u, v, px, py):
    if u[0] < v[0] or (u[0] == v[0] and u[1] < v[1]):
        return (v[0] - u[0]) * (py - u[1]) - (v[1] - u[1]) * (px - u[0])
    return -((u[0] - v[0]) * (py - v[1]) - (u[1] - v[1]) * (px - v[0]))


def _edge_in(e, u, v):
    dy = v[1] - u[1]
    if dy != 0.0:
        tie = dy < 0.0
    else:
        tie = v[0] - u[0] > 0.0
    return np.where(e != 0.0, e > 0.0, tie)


def _centres_below(z, oz, voxel, k0, k1):
    t = (z - oz) / voxel - 0.5
    k = np.where(~(t > k0), k0, np.where(~(t < k1), k1, np.ceil(np.where(np.isfinite(t), t, 0.0)))).astype(np.int64)
    for _ in range(4):
        down = (k > k0) & (oz + ((k - 1).astype(np.float64) + 0.5) * voxel >= z)
        k = np.where(down, k - 1, k)
    for _ in range(4):
        up = (k < k1) & (oz + (k.astype(np.float64) + 0.5) * voxel < z)
        k = np.where(up, k + 1, k)
    return k - k0


def voxelize_mesh(vertices, triangles, matrix, dims, voxel, origin, grid=None):
    """OR one mesh's occupancy into `grid` (uint8, (nz, ny, nx)); returns it."""
    nx, ny, nz = (int(d) for d in dims)
    if grid is None:
        grid = np.zeros((nz, ny, nx), np.uint8)
    tri = np.asarray(triangles, np.int64).reshape(-1, 3)
    verts = np.asarray(vertices, np.float32).reshape(-1, 3)
    if len(verts) == 0 or len(tri) == 0:
        return grid
    m = np.asarray(matrix, np.float32).reshape(4, 4).astype(np.float64)
    a = m[:3, :3]
    det = a[0, 0] * (a[1, 1] * a[2, 2] - a[1, 2] * a[2, 1]) - a[0, 1] * (a[1, 0] * a[2, 2] - a[1, 2] * a[2, 0]) + \
        a[0, 2] * (a[1, 0] * a[2, 1] - a[1, 1] * a[2, 0])
    if det == 0.0:
        return grid
    lo, hi = index_range(verts, matrix, dims, voxel, origin)
    if lo[0] >= hi[0] or lo[1] >= hi[1] or lo[2] >= hi[2]:
        return grid
    w = world_vertices(verts, matrix)
    vox = float(np.float32(voxel))
    ox, oy, oz = (float(np.float32(x)) for x in origin)
    ii, jj = np.meshgrid(np.arange(lo[0], hi[0]), np.arange(lo[1], hi[1]), indexing="xy")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    px = ox + (ii.astype(np.float64) + 0.5) * vox
    py = oy + (jj.astype(np.float64) + 0.5) * vox
    k0, k1 = lo[2], hi[2]
    nzr = k1 - k0
    flips = np.zeros((ii.size, nzr + 1), np.uint8)
    cols = np.arange(ii.size)
    for t in range(len(tri)):
        A, B, C = w[tri[t, 0]].copy(), w[tri[t, 1]].copy(), w[tri[t, 2]].copy()
        sel = ~((px < min(A[0], B[0], C[0])) | (px > max(A[0], B[0], C[0])) | (py < min(A[1], B[1], C[1])) |
                (py > max(A[1], B[1], C[1])))
        if not sel.any():
            continue
        area = (B[0] - A[0]) * (C[1] - A[1]) - (B[1] - A[1]) * (C[0] - A[0])
        if area == 0.0:
            continue
        if area < 0.0:
            B, C = C, B
        qx, qy, qc = px[sel], py[sel], cols[sel]
        wa = _edge_fn(B, C, qx, qy)
        wb = _edge_fn(C, A, qx, qy)
        wc = _edge_fn(A, B, qx, qy)
        ins = _edge_in(wa, B, C) & _edge_in(wb, C, A) & _edge_in(wc, A, B)
        if not ins.any():
            continue
        wa, wb, wc, qc = wa[ins], wb[ins], wc[ins], qc[ins]
        z = ((wa * A[2] + wb * B[2]) + wc * C[2]) / ((wa + wb) + wc)
        mi = _centres_below(z, oz, vox, k0, k1)
        np.bitwise_xor.at(flips, (qc, mi), 1)
    inside = np.bitwise_xor.accumulate(flips[:, :0:-1], axis=1)[:, ::-1]  # inside[:, r] = xor of flips[:, r+1:]
    ks = np.arange(k0, k1)
    occ = inside.astype(bool)
    for r in range(nzr):
        hit = occ[:, r]
        if hit.any():
            grid[ks[r], jj[hit], ii[hit]] = 1
    return grid


def voxelize_meshes(meshes, dims, voxel, origin):
    """The union over (vertices, triangles, matrix) meshes."""
    nx, ny, nz = (int(d) for d in dims)
    grid = np.zeros((nz, ny, nx), np.uint8)
    for verts, tris, matrix in meshes:
        voxelize_mesh(verts, tris, matrix, dims, voxel, origin, grid)
    return grid
