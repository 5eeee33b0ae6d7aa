"""How far a substep's float32 result moves under the smallest change of its
inputs: the yardstick for arithmetic that rounds differently from the oracle.

A one-substep PBF map can be ill-conditioned. From a seeded lattice the
cohesion term drives interior particles to the speed clamp along n/|n|, where
n is a cancelling sum. Near a collider the push-out picks the nearest free
voxel, a discontinuous choice. At a cell boundary the 27-cell stencil
follows the particle's current cell. There, changing every input position by
one ulp already moves the oracle's own output by more than 1e-5 h. Any
float32 evaluation that rounds differently (the GPU's FAST arithmetic, or the
reference's own GLSL in a different within-cell order) moves it by the same
kind of amount. EXACT is held to bit-exactness instead. FAST is held to the
1e-5 h bar where the substep is well conditioned. Elsewhere it is held to
within a small factor of this sensitivity, quantile by quantile.
"""

from __future__ import annotations

import numpy as np

QUANTILES = (0.5, 0.9, 0.99, 0.999)


def ulp_neighbour(positions, seed=0):
    """Every coordinate moved by -1, 0 or +1 ulp (uniformly at random)."""
    rng = np.random.default_rng(seed)
    p = np.asarray(positions, np.float32)
    step = rng.integers(-1, 2, size=p[:, :3].shape)
    out = p.copy()
    target = np.where(step > 0, np.inf, np.where(step < 0, -np.inf, p[:, :3])).astype(np.float32)
    out[:, :3] = np.nextafter(p[:, :3], target)
    return out


def perturbed_state(state, seed=0):
    """The state with every input position - positions and predicted
    positions - moved by -1, 0 or +1 ulp per coordinate."""
    out = dict(state)
    out["positions"] = ulp_neighbour(state["positions"], seed)
    out["predicted"] = ulp_neighbour(state["predicted"], seed + 1)
    return out


def per_particle(a, b, h):
    """max |a - b| over x, y, z per particle, in units of h."""
    return np.abs(np.asarray(a)[:, :3].astype(np.float64) - np.asarray(b)[:, :3]).max(axis=1) / h


def summary(err):
    return {"max": float(err.max()), **{f"q{q}": float(np.quantile(err, q)) for q in QUANTILES},
            "over_1e-5h": int((err > 1e-5).sum())}


def assert_within_sensitivity(tag, err, noise, factor=4.0, floor=1e-6):
    """err (|FAST - oracle|) no worse than `factor` x the oracle's own 1-ulp
    sensitivity at each quantile (plus `floor` h, a few float32 ulps of a
    unit-h coordinate), and no more particles above 1e-5 h than `factor` x
    the sensitivity's count (plus 16)."""
    e, s = summary(err), summary(noise)
    print(f"{tag}: |FAST - oracle| {fmt(e)}; oracle 1-ulp sensitivity {fmt(s)}")
    for q in QUANTILES:
        k = f"q{q}"
        assert e[k] <= factor * s[k] + floor, (tag, k, e[k], s[k])
    assert e["over_1e-5h"] <= factor * s["over_1e-5h"] + 16, (tag, e["over_1e-5h"], s["over_1e-5h"])
    return e, s


def fmt(d):
    return ", ".join(f"{k} {v:.2e}" if isinstance(v, float) else f"{k} {v}" for k, v in d.items())
