"""CPU restatement of the reference's marching cubes (test infrastructure).

Follows solver/marching_cubes.py of Flow-X:

* ``case_table()`` - the 256-case triangle table, derived from the cube's
  geometry the way ``_build_case_table`` (:122-164) derives it: faces wound
  counterclockwise seen from outside (:76-89), per face the directed contour
  segments that pair each inside->outside corner step with the next
  outside->inside step (:92-119), the segments chained into loops, and each
  loop fan-triangulated in reverse;
* ``extract(field, dims, origin, spacing, iso)`` - ``extract`` (:191-280),
  vectorised with NumPy but with the reference's output exactly: cubes in
  (k, j, i) order, triangles in table order, one vertex per crossed lattice
  edge numbered by first use, coordinates in float64 evaluated with the
  reference's expressions (``origin + (i + dx) * spacing``, then
  ``+ t * spacing`` along the edge's axis, ``t = (iso - lo) / (hi - lo)`` or
  0.5 when the two samples are equal).

Pinned against the reference's own table and meshes stored in
tests/golden/mc_golden.npz. Only the tests and the CPU baseline of bench.py
use this module; the product's extraction runs on the GPU.
"""

from __future__ import annotations

import numpy as np

CORNERS = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))
EDGES = ((0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7))
FACE_QUADS = ((0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (3, 2, 6, 7), (0, 3, 7, 4), (1, 2, 6, 5))


def _outward_faces():
    """Each face quad wound counterclockwise seen from outside the cube: the
    Newell normal of the quad must point along (face centre - cube centre)."""
    out = []
    for quad in FACE_QUADS:
        pts = np.array([CORNERS[c] for c in quad], np.float64)
        nxt = np.roll(pts, -1, axis=0)
        normal = np.array([
            ((pts[:, 1] - nxt[:, 1]) * (pts[:, 2] + nxt[:, 2])).sum(),
            ((pts[:, 2] - nxt[:, 2]) * (pts[:, 0] + nxt[:, 0])).sum(),
            ((pts[:, 0] - nxt[:, 0]) * (pts[:, 1] + nxt[:, 1])).sum(),
        ])
        centre = pts.mean(axis=0) - 0.5
        out.append(quad if float(normal @ centre) > 0.0 else quad[::-1])
    return out


def _edge_index(a, b):
    for e, (p, q) in enumerate(EDGES):
        if {p, q} == {a, b}:
            return e
    raise KeyError((a, b))


def case_table():
    """(table, counts): table[case] holds counts[case] triangles as edge
    triples, -1 padded to 15 entries."""
    faces = _outward_faces()
    table = np.full((256, 15), -1, np.int32)
    counts = np.zeros(256, np.int32)
    for case in range(256):
        inside = [(case >> c) & 1 == 1 for c in range(8)]
        succ = {}
        for face in faces:
            steps = []  # (opens, edge) along the face's winding
            for n, a in enumerate(face):
                b = face[(n + 1) % 4]
                if inside[a] != inside[b]:
                    steps.append((inside[a], _edge_index(a, b)))
            for n, (opens, edge) in enumerate(steps):
                if not opens:
                    continue
                for m in range(1, len(steps)):
                    closes, other = steps[(n + m) % len(steps)]
                    if not closes:
                        succ[edge] = other
                        break
        tris = []
        seen = set()
        for first in succ:  # insertion order, as the reference's dict walk
            if first in seen:
                continue
            loop, e = [], first
            while e not in seen:
                seen.add(e)
                loop.append(e)
                e = succ[e]
            for m in range(1, len(loop) - 1):
                tris.append((loop[0], loop[m + 1], loop[m]))
        counts[case] = len(tris)
        for t, tri in enumerate(tris):
            table[case, 3 * t:3 * t + 3] = tri
    return table, counts


def _edge_walk():
    """Per edge: (lower corner, upper corner, axis), the lower corner being
    the one with the smaller coordinate along the edge's axis."""
    walk = []
    for a, b in EDGES:
        axis = next(i for i in range(3) if CORNERS[a][i] != CORNERS[b][i])
        walk.append((a, b, axis) if CORNERS[a][axis] < CORNERS[b][axis] else (b, a, axis))
    return np.array(walk, np.int64)


_TABLE = None


def extract(field, dims, origin, spacing, iso):
    """(vertices float64 V x 3, triangles int32 T x 3), identical to the
    reference's extract on the same samples (the samples indexed
    (k * ny + j) * nx + i; samples >= iso are inside)."""
    global _TABLE
    if _TABLE is None:
        _TABLE = case_table()
    table, counts = _TABLE
    nx, ny, nz = (int(d) for d in dims)
    if nx < 2 or ny < 2 or nz < 2:
        return np.zeros((0, 3), np.float64), np.zeros((0, 3), np.int32)
    f = np.asarray(field).reshape(-1).astype(np.float64)
    iso = float(iso)
    spacing = float(spacing)
    inside = (f >= iso).reshape(nz, ny, nx)
    case = np.zeros((nz - 1, ny - 1, nx - 1), np.int32)
    for c, (dx, dy, dz) in enumerate(CORNERS):
        case |= inside[dz:nz - 1 + dz, dy:ny - 1 + dy, dx:nx - 1 + dx].astype(np.int32) << c
    case = case.reshape(-1)
    cubes = np.nonzero((case != 0) & (case != 255))[0]
    if cubes.size == 0:
        return np.zeros((0, 3), np.float64), np.zeros((0, 3), np.int32)
    ccase = case[cubes]
    per = counts[ccase] * 3
    total = int(per.sum())
    owner = np.repeat(np.arange(cubes.size), per)
    start = np.cumsum(per) - per
    slot = np.arange(total) - np.repeat(start, per)
    edge = table[ccase[owner], slot]
    # the cube's lattice corner 0 and the referenced edge's lower corner
    cube = cubes[owner]
    ci = cube % (nx - 1)
    cj = (cube // (nx - 1)) % (ny - 1)
    ck = cube // ((nx - 1) * (ny - 1))
    walk = _edge_walk()
    lo_corner = walk[edge, 0]
    axis = walk[edge, 2]
    corner = np.array(CORNERS, np.int64)
    li = ci + corner[lo_corner, 0]
    lj = cj + corner[lo_corner, 1]
    lk = ck + corner[lo_corner, 2]
    lattice = (lk * ny + lj) * nx + li
    key = lattice * 3 + axis
    uniq, first, inverse = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # vertices by first use
    rank = np.empty(uniq.size, np.int64)
    rank[order] = np.arange(uniq.size)
    triangles = rank[inverse.reshape(-1)].reshape(-1, 3).astype(np.int32)
    vkey = uniq[order]
    vaxis = vkey % 3
    vlat = vkey // 3
    vi = vlat % nx
    vj = (vlat // nx) % ny
    vk = vlat // (nx * ny)
    stride = np.array([1, nx, nx * ny], np.int64)[vaxis]
    lo = f[vlat]
    hi = f[vlat + stride]
    delta = hi - lo
    zero = delta == 0.0
    t = np.where(zero, 0.5, (iso - lo) / np.where(zero, 1.0, delta))
    ox, oy, oz = (float(v) for v in origin)
    pts = np.stack([ox + vi.astype(np.float64) * spacing,
                    oy + vj.astype(np.float64) * spacing,
                    oz + vk.astype(np.float64) * spacing], axis=1)
    rows = np.arange(pts.shape[0])
    pts[rows, vaxis] = pts[rows, vaxis] + t * spacing
    return pts, triangles
