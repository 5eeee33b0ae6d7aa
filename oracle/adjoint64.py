"""Oracle (test infrastructure only): float64 torch re-expression of the PBF
substep, differentiated by torch autograd, against which the library's
hand-written adjoint (flowx_substep_adjoint) is checked. Never imported by
the product path.

The passes are those of oracle/ref64.py, which restates the reference's GLSL
passes (shaders/sph_normal.glsl, sph_predict.glsl, sph_lambda.glsl,
sph_delta.glsl, sph_apply_delta.glsl, sph_velocity.glsl, sph_xsph.glsl,
sph_finalize.glsl, surface_splat.glsl; the sequence of solver/sph.py:501-514)
with the same neighbour semantics. Each pass's candidate pairs come from
``ref64.pairs`` on the current positions against the substep's grid, found
without gradients, the way the library's adjoint holds the grid and the
candidate sets fixed; the r < h, r^2 > 1e-12, j != i and clamp selections are
masks of the current values. All arithmetic on positions, velocities and
densities is differentiable.

The candidate search is the brute-force pair enumeration of ``ref64.pairs``
(every particle against every slot of its 27 cells); at the sizes the tests
use (about 2,000 particles) that is the dense reference.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ref64 as R

F64 = torch.float64


def params(config, dt, collider=None, collider_voxel=0.0):
    """ref64.Params of a flowx_gb300.config.SolverConfig."""
    c = config
    return R.Params(lo=c.lo, hi=c.hi, cell_size=c.cell_size, cell_dims=c.cell_dims, h=c.smoothing_radius,
                    mass=c.mass, rest_density=c.rest_density, relaxation=c.relaxation, scorr=c.scorr_strength,
                    sigma=c.surface_tension, viscosity=c.viscosity, dt=dt, particle_radius=c.particle_radius,
                    collider=collider, collider_voxel=collider_voxel)


def _pairs(p, grid, prm, radius=1):
    keys, cs, ce = grid
    q = p.detach().cpu().numpy()
    i, j = R.pairs(q, keys, cs, ce, prm, radius)
    return torch.as_tensor(i), torch.as_tensor(j)


def _sum(i, v, n):
    out = torch.zeros((n,) + tuple(v.shape[1:]), dtype=v.dtype)
    return out.index_add(0, i, v)


def _norm(v):
    return torch.sqrt((v * v).sum(1))


def _safe_sqrt(x):
    pos = x > 0
    return torch.where(pos, torch.sqrt(torch.where(pos, x, torch.ones_like(x))), torch.zeros_like(x))


def normal(p, rho, grid, prm):
    """sph_normal.glsl over the previous substep's grid: (normal, curvature)."""
    n = p.shape[0]
    i, j = _pairs(p, grid, prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = (d * d).sum(1)
    h, h2 = prm.h, prm.h * prm.h
    keep = (r2 < h2).detach()
    i, j, d, r2 = i[keep], j[keep], d[keep], r2[keep]
    w = prm.mass / torch.clamp(rho[j], min=1e-6)
    t = h2 - r2
    grad = (R.poly6_coef(h) * -6.0 * t * t)[:, None] * d
    nrm = _sum(i, w[:, None] * grad, n)
    lap = _sum(i, w * R.visc_lap_coef(h) * (h - _safe_sqrt(r2)), n)
    mag = _norm(nrm)
    m = (mag > 1e-4).detach()
    curv = torch.where(m, -lap / torch.where(m, mag, torch.ones_like(mag)), torch.zeros_like(lap))
    return nrm, curv


def predict(pos, vel, nrm, curv, prm):
    """sph_predict.glsl: gravity, cohesion, speed clamp, predicted position."""
    dt = prm.dt
    v = vel + torch.tensor([0.0, 0.0, prm.g * dt], dtype=F64)
    if prm.sigma > 0.0:
        mag = _norm(nrm)
        m = (mag > 1e-4).detach()
        safe = torch.where(m, mag, torch.ones_like(mag))
        add = ((-prm.sigma * curv / safe / prm.mass)[:, None] * nrm) * dt
        v = v + torch.where(m[:, None], add, torch.zeros_like(add))
    vmax = 0.4 * prm.h / max(dt, 1e-6)
    speed = _norm(v)
    s = (speed > vmax).detach()
    v = torch.where(s[:, None], v * (vmax / torch.where(s, speed, torch.ones_like(speed)))[:, None], v)
    return pos + v * dt


def lambda_pass(p, grid, prm):
    """sph_lambda.glsl: (max(density, 1e-6), lambda)."""
    n = p.shape[0]
    i, j = _pairs(p, grid, prm)
    d = p[i] - p[j]
    r2 = (d * d).sum(1)
    h, h2 = prm.h, prm.h * prm.h
    inside = (r2 < h2).detach()
    t = torch.where(inside, h2 - r2, torch.zeros_like(r2))
    density = _sum(i, prm.mass * R.poly6_coef(h) * t**3, n)
    g = ((j != i) & inside & (r2 > 1e-12)).detach()
    ig, dg = i[g], d[g]
    r = torch.sqrt((dg * dg).sum(1))
    grad = (prm.mass * R.spiky_grad_coef(h) * (h - r) ** 2 / r)[:, None] * dg
    gs = _sum(ig, grad, n)
    gn = _sum(ig, (grad * grad).sum(1), n)
    rho = torch.clamp(density, min=1e-6)
    c = rho / prm.rho0 - 1.0
    denom = ((gs * gs).sum(1) + gn) / (prm.rho0 * prm.rho0) + prm.eps
    lam = -c / torch.clamp(denom, min=1e-9)
    return rho, lam


def delta_pass(p, lam, grid, prm):
    """sph_delta.glsl: the position correction."""
    n = p.shape[0]
    i, j = _pairs(p, grid, prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = (d * d).sum(1)
    h, h2 = prm.h, prm.h * prm.h
    keep = ((r2 < h2) & (r2 > 1e-12)).detach()
    i, j, d, r2 = i[keep], j[keep], d[keep], r2[keep]
    r = torch.sqrt(r2)
    coef = R.poly6_coef(h)
    wq = coef * (h2 - (0.2 * h) ** 2) ** 3 if (0.2 * h) ** 2 < h2 else 0.0
    scorr = torch.zeros_like(r)
    if prm.scorr > 0.0 and wq > 1e-9:
        ratio = coef * (h2 - r2) ** 3 / wq
        scorr = -prm.scorr * torch.clamp(ratio, min=0.0) ** 4
    term = ((lam[i] + lam[j] + scorr) * R.spiky_grad_coef(h) * (h - r) ** 2 / r)[:, None] * d
    return _sum(i, term, n) / prm.rho0


def xsph(p, v, rho, grid, prm):
    """sph_xsph.glsl: c sum (m / rho_j)(v_j - v_i) W."""
    n = p.shape[0]
    i, j = _pairs(p, grid, prm)
    keep = j != i
    i, j = i[keep], j[keep]
    d = p[i] - p[j]
    r2 = (d * d).sum(1)
    h2 = prm.h * prm.h
    keep = (r2 < h2).detach()
    i, j, r2 = i[keep], j[keep], r2[keep]
    w = prm.mass / torch.clamp(rho[j], min=1e-6) * R.poly6_coef(prm.h) * (h2 - r2) ** 3
    return prm.visc * _sum(i, w[:, None] * (v[j] - v[i]), n)


def _collider_targets(p_np, prm):
    """Per particle: the nearest free voxel centre of sph_finalize.glsl's search
    (NaN where the particle is outside the collider or none is free)."""
    out = np.full(p_np.shape, np.nan)
    if prm.collider is None or prm.voxel <= 0.0:
        return out
    c = np.floor((p_np - prm.lo) / prm.voxel).astype(np.int64)
    inside, _ = R._occupied(c, prm)
    rng = range(-R.MAX_COLLIDER_SEARCH, R.MAX_COLLIDER_SEARCH + 1)
    for idx in np.nonzero(inside)[0]:
        best, best_d2 = None, 1e30
        for dz in rng:
            for dy in rng:
                for dx in rng:
                    nc = c[idx] + np.array([dx, dy, dz])
                    occ, inb = R._occupied(nc[None, :], prm)
                    if not inb[0] or occ[0]:
                        continue
                    centre = prm.lo + (nc + 0.5) * prm.voxel
                    d2 = float(np.dot(centre - p_np[idx], centre - p_np[idx]))
                    if d2 < best_d2:
                        best_d2, best = d2, centre
        if best is not None:
            out[idx] = best
    return out


def finalize(p, v, prm):
    """sph_finalize.glsl: collider push-out, then the box clamp with damping."""
    targets = torch.as_tensor(_collider_targets(p.detach().numpy(), prm))
    hit = ~torch.isnan(targets[:, 0])
    if bool(hit.any()):
        best = torch.where(hit[:, None], targets, torch.zeros_like(targets))
        e = best - p
        dist = _norm(e)
        far = (dist > 1e-6).detach()
        u = torch.where((hit & far)[:, None], e / torch.where(far, dist, torch.ones_like(dist))[:, None],
                        torch.tensor([0.0, 0.0, 1.0], dtype=F64).expand_as(e))
        p = torch.where(hit[:, None], p + u * (dist + prm.radius)[:, None], p)
        vn = (v * u).sum(1)
        neg = (hit & (vn < 0.0)).detach()
        v = torch.where(neg[:, None], v - (vn * (1.0 + prm.damping))[:, None] * u, v)
    lo = torch.as_tensor(prm.lo + prm.radius)
    hi = torch.as_tensor(prm.hi - prm.radius)
    below = (p < lo).detach()
    above = (~below & (p > hi)).detach()
    p = torch.where(below, lo.expand_as(p), torch.where(above, hi.expand_as(p), p))
    v = torch.where(below | above, -v * prm.damping, v)
    return p, v


def splat(pos, grid, prm, surface):
    """surface_splat.glsl: density / rho0 at every splat sample."""
    nx, ny, nz = surface.dims
    s = np.arange(nx * ny * nz)
    g = np.stack([s % nx, (s // nx) % ny, s // (nx * ny)], axis=1)
    pts = np.asarray(surface.lo, dtype=np.float64) + g * surface.spacing
    keys, cs, ce = grid
    i, j = R.pairs(pts, keys, cs, ce, prm, radius=2)
    i, j = torch.as_tensor(i), torch.as_tensor(j)
    d = torch.as_tensor(pts)[i] - pos[j]
    r2 = (d * d).sum(1)
    kr = surface.kernel_radius
    h2 = kr * kr
    inside = (r2 < h2).detach()
    t = torch.where(inside, h2 - r2, torch.zeros_like(r2))
    value = _sum(i, prm.mass * R.poly6_coef(kr) * t**3, pts.shape[0]) / max(prm.rho0, 1e-6)
    if prm.collider is not None and prm.voxel > 0.0:
        c = np.floor((pts - prm.lo) / prm.voxel).astype(np.int64)
        occ, _ = R._occupied(c, prm)
        value = value * torch.as_tensor(~occ, dtype=F64)
    return value


def _grid(q, prm, sorted_count):
    return R.build_grid(q.detach().numpy(), prm, sorted_count)


def substep(state, grid_prev, prm, sorted_count, iterations, grid=None):
    """One substep (solver/sph.py:501-514) on float64 tensors; returns the next
    state and the grid it built (or was given)."""
    pos, vel, pred, rho = state["positions"], state["velocities"], state["predicted"], state["density"]
    if prm.sigma > 0.0:
        nrm, curv = normal(pred, rho, grid_prev, prm)
    else:
        nrm = torch.zeros_like(pos)
        curv = torch.zeros(pos.shape[0], dtype=F64)
    q = predict(pos, vel, nrm, curv, prm)
    if grid is None:
        grid = _grid(q, prm, sorted_count)
    p = q
    rho_last = None
    for _ in range(iterations):
        rho_last, lam = lambda_pass(p, grid, prm)
        p = p + delta_pass(p, lam, grid, prm)
    v = (p - pos) / max(prm.dt, 1e-6)
    v = v + xsph(p, v, rho_last, grid, prm)
    pos2, vel2 = finalize(p, v, prm)
    return {"positions": pos2, "velocities": vel2, "predicted": p, "density": rho_last}, grid


def rollout(pos0, vel0, prm, sorted_count, iterations, substeps, surface=None):
    """``substeps`` substeps from (pos0, vel0) ((N, 3) float64 tensors) from the
    state _allocate and _seed leave (predicted = positions, densities zero,
    grid from positions); returns (splat or None, final state)."""
    grid = _grid(pos0, prm, sorted_count)
    state = {"positions": pos0, "velocities": vel0, "predicted": pos0,
             "density": torch.zeros(pos0.shape[0], dtype=F64)}
    for _ in range(substeps):
        state, grid = substep(state, grid, prm, sorted_count, iterations)
    surf = splat(state["positions"], grid, prm, surface) if surface is not None else None
    return surf, state


def _pin(value, carrier):
    """``value`` as the forward value, with ``carrier``'s gradient path."""
    return torch.as_tensor(np.asarray(value, dtype=np.float64)) + (carrier - carrier.detach())


def rollout_along(pos0, vel0, prm, sorted_count, iterations, states, grids, surface=None):
    """The rollout of ``rollout`` with every substep's Jacobian evaluated at a
    given trajectory: ``states[s]`` holds the (positions, velocities, predicted,
    density) arrays entering substep s (s = 0..S, S = len(states) - 1) and
    ``grids[s]`` the grid of substep s's normal pass (``grids[s + 1]`` is the
    grid substep s builds). Forward values are those of the given trajectory
    (for instance the float32 oracle's), gradients flow through the float64
    passes, so autograd returns the float64 adjoint of that trajectory, which
    the library's float32 adjoint approximates over any horizon, however far
    float32 and float64 forwards drift apart."""
    cur = {"positions": pos0, "velocities": vel0, "predicted": pos0,
           "density": torch.zeros(pos0.shape[0], dtype=F64)}
    nsub = len(states) - 1
    for s in range(nsub):
        st = {k: _pin(states[s][k], cur[k]) for k in cur}
        cur, _ = substep(st, grids[s], prm, sorted_count, iterations, grid=grids[s + 1])
    final = {k: _pin(states[nsub][k], cur[k]) for k in ("positions", "velocities")}
    surf = splat(final["positions"], grids[nsub], prm, surface) if surface is not None else None
    return surf, final


def central_difference(fn, x: torch.Tensor, direction: torch.Tensor, eps=1e-4) -> float:
    """(fn(x + eps u) - fn(x - eps u)) / (2 eps) in float64."""
    with torch.no_grad():
        return float((fn(x + eps * direction) - fn(x - eps * direction)) / (2.0 * eps))


__all__ = ["params", "rollout", "rollout_along", "substep", "central_difference"]
