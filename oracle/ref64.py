"""Oracle (test infrastructure only): float64 NumPy re-expression of the PBF passes.

Each function restates one reference pass over whole arrays, in float64, with
the reference's neighbour semantics: candidates come from the 3x3x3 (splat:
5x5x5) cells around ``clamp(floor((p - lo) / cell))`` of the *current* query
position, looked up in the given (possibly stale) key/cell arrays, each cell
scanned for at most MAX_CELL_SCAN entries in key-array order.

Used to state the error of the float32 paths (the GLSL harness, the C
restatement and the CUDA kernels) against exact-ish arithmetic. Buffers use
the reference's layouts: (N, 4) particle arrays, (S, 4) keys (key, id, 0, 0),
(C,) float cell_start / cell_end with -1 for empty.

Reference passes restated here:
  normal        shaders/sph_normal.glsl:24-81
  predict       shaders/sph_predict.glsl:23-57
  grid_key      shaders/sph_grid_key.glsl:14-28
  sort          shaders/sph_sort.glsl:14-34 (as a stable key sort; see below)
  cell ranges   shaders/sph_cell_clear.glsl:8-16, sph_cell_range.glsl:10-32
  lambda        shaders/sph_lambda.glsl:17-77
  delta         shaders/sph_delta.glsl:19-85
  apply_delta   shaders/sph_apply_delta.glsl:10-20
  velocity      shaders/sph_velocity.glsl:12-24
  xsph          shaders/sph_xsph.glsl:28-82
  finalize      shaders/sph_finalize.glsl:13-96
  splat         shaders/surface_splat.glsl:30-97
with the kernels of shaders/sph_common.glsl:66-127.
"""

from __future__ import annotations

import math

import numpy as np

MAX_CELL_SCAN = 512
MAX_COLLIDER_SEARCH = 2


class Params:
    """The push-block fields the passes read, as float64 scalars."""

    def __init__(self, *, lo, hi, cell_size, cell_dims, h, mass, rest_density, relaxation, scorr, sigma,
                 viscosity, dt, particle_radius, gravity=-9.81, damping=0.35, collider=None, collider_voxel=0.0):
        self.lo = np.asarray(lo, dtype=np.float64)
        self.hi = np.asarray(hi, dtype=np.float64)
        self.cell = float(cell_size)
        self.dims = np.asarray(cell_dims, dtype=np.int64)
        self.h, self.mass, self.rho0, self.eps = float(h), float(mass), float(rest_density), float(relaxation)
        self.scorr, self.sigma, self.visc, self.dt = float(scorr), float(sigma), float(viscosity), float(dt)
        self.radius, self.g, self.damping = float(particle_radius), float(gravity), float(damping)
        self.collider = None if collider is None else (np.asarray(collider) > 0)
        self.voxel = float(collider_voxel)


def poly6_coef(h):
    return 315.0 / (64.0 * math.pi * h**9)


def spiky_grad_coef(h):
    return -45.0 / (math.pi * h**6)


def visc_lap_coef(h):
    return 45.0 / (math.pi * h**6)


def cell_coord(p, prm):
    g = np.floor((p[:, :3] - prm.lo) / prm.cell).astype(np.int64)
    return np.clip(g, 0, prm.dims - 1)


def cell_index(g, dims):
    return (g[:, 2] * dims[1] + g[:, 1]) * dims[0] + g[:, 0]


def pairs(query, keys, cell_start, cell_end, prm, radius=1):
    """Candidate pairs (i, j) in the reference's visiting order.

    For every query point, the (2r+1)^3 cells around its clamped cell coordinate
    in dz, dy, dx order, each scanned from cell_start for at most MAX_CELL_SCAN
    key slots. Returns (i, j) int64 arrays.
    """
    base = cell_coord(query, prm)
    ids = keys[:, 1].astype(np.int64)
    cs = cell_start.astype(np.int64)
    ce = cell_end.astype(np.int64)
    nq = query.shape[0]
    parts_i, parts_k, parts_o = [], [], []
    order = 0
    for dz in range(-radius, radius + 1):
        for dy in range(-radius, radius + 1):
            for dx in range(-radius, radius + 1):
                g = base + np.array([dx, dy, dz])
                ok = np.all((g >= 0) & (g < prm.dims), axis=1)
                qi = np.nonzero(ok)[0]
                c = cell_index(g[qi], prm.dims)
                start = cs[c]
                ok2 = start >= 0
                qi, start, c = qi[ok2], start[ok2], c[ok2]
                end = np.minimum(ce[c], start + MAX_CELL_SCAN)
                cnt = np.maximum(end - start, 0)
                rep_i = np.repeat(qi, cnt)
                offs = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
                parts_i.append(rep_i)
                parts_k.append(np.repeat(start, cnt) + offs)
                parts_o.append(np.full(rep_i.shape, order))
                order += 1
    i = np.concatenate(parts_i) if parts_i else np.zeros(0, np.int64)
    k = np.concatenate(parts_k) if parts_k else np.zeros(0, np.int64)
    o = np.concatenate(parts_o) if parts_o else np.zeros(0, np.int64)
    perm = np.lexsort((k, o, i))
    i, k = i[perm], k[perm]
    return i, ids[k]


def _sum(i, values, n):
    out = np.zeros((n,) + values.shape[1:], dtype=np.float64)
    np.add.at(out, i, values)
    return out


def normal(st, prm):
    p = st["predicted"][:, :3].astype(np.float64)
    n = p.shape[0]
    i, j = pairs(p, st["keys"], st["cell_start"], st["cell_end"], prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = np.einsum("ij,ij->i", d, d)
    h2 = prm.h * prm.h
    keep = r2 < h2
    i, j, d, r2 = i[keep], j[keep], d[keep], r2[keep]
    rho_j = np.maximum(st["lambda"][j, 0].astype(np.float64), 1e-6)
    w = prm.mass / rho_j
    t = h2 - r2
    grad = (poly6_coef(prm.h) * -6.0 * t * t)[:, None] * d
    nrm = _sum(i, w[:, None] * grad, n)
    lap = _sum(i, w * visc_lap_coef(prm.h) * (prm.h - np.sqrt(r2)), n)
    mag = np.linalg.norm(nrm, axis=1)
    curv = np.where(mag > 1e-4, -lap / np.where(mag > 1e-4, mag, 1.0), 0.0)
    out = np.zeros((n, 4))
    out[:, :3] = nrm
    out[:, 3] = curv
    return out


def predict(st, prm):
    v = st["velocities"][:, :3].astype(np.float64).copy()
    dt = prm.dt
    v[:, 2] += prm.g * dt
    if prm.sigma > 0.0:
        nrm = st["normal"].astype(np.float64)
        mag = np.linalg.norm(nrm[:, :3], axis=1)
        m = mag > 1e-4
        safe = np.where(m, mag, 1.0)
        v[m] += ((-prm.sigma * nrm[m, 3] / safe[m] / prm.mass)[:, None] * nrm[m, :3]) * dt
    vmax = 0.4 * prm.h / max(dt, 1e-6)
    speed = np.linalg.norm(v, axis=1)
    s = speed > vmax
    v[s] *= (vmax / speed[s])[:, None]
    p = st["positions"][:, :3].astype(np.float64) + v * dt
    vel = np.zeros((v.shape[0], 4))
    vel[:, :3] = v
    pred = np.ones((v.shape[0], 4))
    pred[:, :3] = p
    return vel, pred


def grid_keys(pred, prm, sorted_count):
    """(key, id) per slot before sorting (sph_grid_key.glsl:14-28)."""
    n = pred.shape[0]
    cell_count = int(np.prod(prm.dims))
    key = np.full(sorted_count, cell_count, dtype=np.int64)
    key[:n] = cell_index(cell_coord(pred, prm), prm.dims)
    return key


def build_grid(pred, prm, sorted_count):
    """Keys sorted by (key, id) and the per-cell [start, end) ranges.

    The reference's bitonic sort (sph_sort.glsl) orders by key only and is not
    stable; this uses the stable (key, id) order. Cell ranges and each cell's
    membership are the same under both.
    """
    key = grid_keys(pred, prm, sorted_count)
    ids = np.arange(sorted_count)
    perm = np.lexsort((ids, key))
    keys = np.zeros((sorted_count, 4))
    keys[:, 0] = key[perm]
    keys[:, 1] = ids[perm]
    cell_count = int(np.prod(prm.dims))
    cs = np.full(cell_count, -1.0)
    ce = np.full(cell_count, -1.0)
    real = keys[:, 0] < cell_count
    kk = keys[real, 0].astype(np.int64)
    slots = np.nonzero(real)[0]
    first = np.r_[True, kk[1:] != kk[:-1]]
    last = np.r_[kk[1:] != kk[:-1], True]
    cs[kk[first]] = slots[first]
    ce[kk[last]] = slots[last] + 1
    return keys, cs, ce


def lambda_pass(st, prm):
    p = st["predicted"][:, :3].astype(np.float64)
    n = p.shape[0]
    i, j = pairs(p, st["keys"], st["cell_start"], st["cell_end"], prm)
    d = p[i] - p[j]
    r2 = np.einsum("ij,ij->i", d, d)
    h2 = prm.h * prm.h
    t = np.maximum(h2 - r2, 0.0)
    density = _sum(i, prm.mass * poly6_coef(prm.h) * t**3 * (r2 < h2), n)
    g = (j != i) & (r2 < h2) & (r2 > 1e-12)
    ig, dg, r = i[g], d[g], np.sqrt(r2[g])
    grad = (prm.mass * spiky_grad_coef(prm.h) * (prm.h - r) ** 2 / r)[:, None] * dg
    gs = _sum(ig, grad, n)
    gn = _sum(ig, np.einsum("ij,ij->i", grad, grad), n)
    rho = np.maximum(density, 1e-6)
    c = rho / prm.rho0 - 1.0
    denom = (np.einsum("ij,ij->i", gs, gs) + gn) / (prm.rho0 * prm.rho0) + prm.eps
    lam = -c / np.maximum(denom, 1e-9)
    out = np.zeros((n, 4))
    out[:, 0] = rho
    out[:, 1] = lam
    return out


def delta_pass(st, prm):
    p = st["predicted"][:, :3].astype(np.float64)
    lam = st["lambda"][:, 1].astype(np.float64)
    n = p.shape[0]
    i, j = pairs(p, st["keys"], st["cell_start"], st["cell_end"], prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = np.einsum("ij,ij->i", d, d)
    h2 = prm.h * prm.h
    keep = (r2 < h2) & (r2 > 1e-12)
    i, j, d, r2 = i[keep], j[keep], d[keep], r2[keep]
    r = np.sqrt(r2)
    coef = poly6_coef(prm.h)
    wq = coef * (h2 - (0.2 * prm.h) ** 2) ** 3 if (0.2 * prm.h) ** 2 < h2 else 0.0
    scorr = np.zeros_like(r)
    if prm.scorr > 0.0 and wq > 1e-9:
        ratio = coef * (h2 - r2) ** 3 / wq
        scorr = -prm.scorr * np.maximum(ratio, 0.0) ** 4
    term = ((lam[i] + lam[j] + scorr) * spiky_grad_coef(prm.h) * (prm.h - r) ** 2 / r)[:, None] * d
    out = np.zeros((n, 4))
    out[:, :3] = _sum(i, term, n) / prm.rho0
    return out


def apply_delta(st):
    out = st["predicted"].astype(np.float64).copy()
    out[:, :3] += st["delta"][:, :3]
    out[:, 3] = 1.0
    return out


def velocity(st, prm):
    v = (st["predicted"][:, :3].astype(np.float64) - st["positions"][:, :3]) / max(prm.dt, 1e-6)
    out = np.zeros((v.shape[0], 4))
    out[:, :3] = v
    return out


def xsph(st, prm):
    p = st["predicted"][:, :3].astype(np.float64)
    v = st["velocities"][:, :3].astype(np.float64)
    n = p.shape[0]
    i, j = pairs(p, st["keys"], st["cell_start"], st["cell_end"], prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = np.einsum("ij,ij->i", d, d)
    h2 = prm.h * prm.h
    keep = r2 < h2
    i, j, r2 = i[keep], j[keep], r2[keep]
    rho_j = np.maximum(st["lambda"][j, 0].astype(np.float64), 1e-6)
    w = prm.mass / rho_j * poly6_coef(prm.h) * (h2 - r2) ** 3
    acc = _sum(i, w[:, None] * (v[j] - v[i]), n)
    out = np.zeros((n, 4))
    out[:, :3] = prm.visc * acc
    return out


def _occupied(c, prm):
    occ = prm.collider
    dims = np.array([occ.shape[2], occ.shape[1], occ.shape[0]])
    inb = np.all((c >= 0) & (c < dims), axis=1)
    out = np.zeros(c.shape[0], dtype=bool)
    cc = c[inb]
    out[inb] = occ[cc[:, 2], cc[:, 1], cc[:, 0]]
    return out, inb


def finalize(st, prm):
    v = st["velocities"][:, :3].astype(np.float64) + st["delta"][:, :3]
    p = st["predicted"][:, :3].astype(np.float64).copy()
    if prm.collider is not None and prm.voxel > 0.0:
        c = np.floor((p - prm.lo) / prm.voxel).astype(np.int64)
        inside, _ = _occupied(c, prm)
        for idx in np.nonzero(inside)[0]:
            best, best_d2 = None, 1e30
            for dz in range(-MAX_COLLIDER_SEARCH, MAX_COLLIDER_SEARCH + 1):
                for dy in range(-MAX_COLLIDER_SEARCH, MAX_COLLIDER_SEARCH + 1):
                    for dx in range(-MAX_COLLIDER_SEARCH, MAX_COLLIDER_SEARCH + 1):
                        nc = c[idx] + np.array([dx, dy, dz])
                        occ, inb = _occupied(nc[None, :], prm)
                        if not inb[0] or occ[0]:
                            continue
                        center = prm.lo + (nc + 0.5) * prm.voxel
                        d2 = float(np.dot(center - p[idx], center - p[idx]))
                        if d2 < best_d2:
                            best_d2, best = d2, center
            if best is not None:
                dist = math.sqrt(best_d2)
                u = (best - p[idx]) / dist if dist > 1e-6 else np.array([0.0, 0.0, 1.0])
                p[idx] += u * (dist + prm.radius)
                vn = float(np.dot(v[idx], u))
                if vn < 0.0:
                    v[idx] -= vn * (1.0 + prm.damping) * u
    lo = prm.lo + prm.radius
    hi = prm.hi - prm.radius
    for a in range(3):
        below = p[:, a] < lo[a]
        above = (~below) & (p[:, a] > hi[a])
        p[below, a] = lo[a]
        p[above, a] = hi[a]
        flip = below | above
        v[flip, a] = -v[flip, a] * prm.damping
    pos = np.ones((p.shape[0], 4))
    pos[:, :3] = p
    vel = np.zeros((p.shape[0], 4))
    vel[:, :3] = v
    return pos, vel


def splat(st, prm, *, dims, spacing, kernel_radius, surface_lo):
    nx, ny, nz = dims
    s = np.arange(nx * ny * nz)
    g = np.stack([s % nx, (s // nx) % ny, s // (nx * ny)], axis=1)
    pts = np.asarray(surface_lo, dtype=np.float64) + g * spacing
    q = np.zeros((pts.shape[0], 4))
    q[:, :3] = pts
    i, j = pairs(q, st["keys"], st["cell_start"], st["cell_end"], prm, radius=2)
    d = pts[i] - st["positions"][j, :3].astype(np.float64)
    r2 = np.einsum("ij,ij->i", d, d)
    h2 = kernel_radius * kernel_radius
    w = np.where(r2 < h2, poly6_coef(kernel_radius) * np.maximum(h2 - r2, 0.0) ** 3, 0.0)
    dens = _sum(i, prm.mass * w, pts.shape[0])
    value = dens / max(prm.rho0, 1e-6)
    if prm.collider is not None and prm.voxel > 0.0:
        c = np.floor((pts - prm.lo) / prm.voxel).astype(np.int64)
        occ, _ = _occupied(c, prm)
        value[occ] = 0.0
    return value


def substep(st, prm, sorted_count, iterations, trace=None):
    """One substep (solver/sph.py:501-514) on a dict of float64 arrays."""
    st = {k: np.asarray(v, dtype=np.float64).copy() for k, v in st.items()}

    def snap(name, **bufs):
        if trace is not None and name not in trace:
            trace[name] = {k: v.copy() for k, v in bufs.items()}

    if prm.sigma > 0.0:
        st["normal"] = normal(st, prm)
        snap("normal", normal=st["normal"])
    st["velocities"], st["predicted"] = predict(st, prm)
    snap("predict", velocities=st["velocities"], predicted=st["predicted"])
    st["keys"], st["cell_start"], st["cell_end"] = build_grid(st["predicted"], prm, sorted_count)
    snap("build_grid", keys=st["keys"], cell_start=st["cell_start"], cell_end=st["cell_end"])
    for _ in range(iterations):
        st["lambda"] = lambda_pass(st, prm)
        snap("lambda", lambda_=st["lambda"])
        st["delta"] = delta_pass(st, prm)
        snap("delta", delta=st["delta"])
        st["predicted"] = apply_delta(st)
        snap("apply_delta", predicted=st["predicted"])
    st["velocities"] = velocity(st, prm)
    snap("velocity", velocities=st["velocities"])
    st["delta"] = xsph(st, prm)
    snap("xsph", delta=st["delta"])
    st["positions"], st["velocities"] = finalize(st, prm)
    snap("finalize", positions=st["positions"], velocities=st["velocities"])
    return st
