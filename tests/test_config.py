"""Host-side restatement (flowx_gb300.config) against the reference's own host
Python, run outside Blender (tests/golden/host_reference.json,
seed_reference.npz)."""

import json
import os

import numpy as np
import pytest

from flowx_gb300 import config as C

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
with open(os.path.join(GOLDEN, "host_reference.json")) as f:
    HOST = json.load(f)


def _resolve(rec):
    d = rec["domain"]
    cfg = C.resolve_config(
        d["lo"], d["hi"], fluid_level=d["fluid_level"], smoothing_radius=d["smoothing_radius"],
        rest_density=d["rest_density"], viscosity=d["viscosity"], relaxation=100.0, scorr_strength=0.1,
        surface_tension=0.05,
    )
    pos = C.seed_positions_reference(cfg, dtype=np.float64)
    cfg.particle_count = pos.shape[0]
    return cfg, pos


@pytest.mark.parametrize("idx", range(len(HOST)))
def test_resolve_config_matches_reference(idx):
    rec = HOST[idx]
    cfg, _ = _resolve(rec)
    want = rec["config"]
    assert cfg.smoothing_radius == want["smoothing_radius"]
    assert cfg.spacing == want["spacing"]
    assert cfg.mass == want["mass"]
    assert cfg.cell_size == want["cell_size"]
    assert list(cfg.cell_dims) == want["cell_dims"]
    assert cfg.cell_count == want["cell_count"]
    assert cfg.particle_count == want["particle_count"]
    assert cfg.sorted_count == want["sorted_count"]


@pytest.mark.parametrize("idx", range(len(HOST)))
def test_substep_dt_matches_reference(idx):
    rec = HOST[idx]
    cfg, _ = _resolve(rec)
    for fps, (steps, dt) in rec["substep_dt"].items():
        got = cfg.substep_dt(1.0 / int(fps))
        assert got[0] == steps and got[1] == dt


@pytest.mark.parametrize("idx", range(len(HOST)))
def test_push_block_matches_reference(idx):
    rec = HOST[idx]
    cfg, _ = _resolve(rec)
    geo = rec["collider_geometry"]
    origin, voxel, dims = C.collider_grid_geometry(rec["domain"]["lo"], rec["domain"]["hi"],
                                                   rec["domain"]["collider_resolution"])
    assert list(origin) == geo["origin"] and voxel == geo["voxel"] and list(dims) == geo["dims"]
    steps, dt = cfg.substep_dt(1.0 / 24)
    got = C.push_constant_values(cfg, dt, C.collider_binding(dims, voxel), 4, 2)
    for name, vec in rec["push"].items():
        assert list(got[name]) == vec, name
    raw = C.pack_push(got)
    assert len(raw) == 128


@pytest.mark.parametrize("idx", range(len(HOST)))
def test_surface_resolve_matches_reference(idx):
    rec = HOST[idx]
    cfg, _ = _resolve(rec)
    surf = C.resolve_surface(cfg, resolution=rec["domain"]["surface_resolution"])
    want = rec["surface"]
    assert list(surf.dims) == want["dims"]
    assert surf.spacing == want["spacing"]
    assert surf.kernel_radius == want["kernel_radius"]
    assert list(surf.lo) == want["lo"]
    assert surf.sample_count == want["sample_count"]


def test_seed_positions_match_reference():
    z = np.load(os.path.join(GOLDEN, "seed_reference.npz"))
    assert z.files
    for key in z.files:
        rec = HOST[int(key[4:])]
        _, pos = _resolve(rec)
        np.testing.assert_array_equal(pos, z[key])
