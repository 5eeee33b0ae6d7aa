"""Crowded neighbourhoods against the oracle, bit for bit (EXACT), one fused
substep after a grid build:

* cells of h with a blob of ~750 particles per cell next to the dam break's
  fluid at rest: stencil rows far over 64 slots (the per-row walk, beside
  lanes on the two-phase walk in the same warps) and cells over the
  reference's MAX_CELL_SCAN = 512 (its per-cell cap,
  shaders/sph_common.glsl:30, sph_lambda.glsl:39-70);
* cells of 2.25 h (the reference's cell rule on the 2 m domain) with one blob
  whose rows exceed MAX_CELL_SCAN and one at ~150 particles per cell, whose
  trimmed rows hold more chunks than the staged walk keeps (both walked again
  in order), beside the fluid's own rows.

Both grid orders: the counting sort's (cell, id) and the reference's bitonic
network."""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BUFS = ("positions", "velocities", "predicted", "lambda", "normal")


def _blob(rng, centre, half, n):
    p = np.zeros((n, 4), np.float32)
    p[:, :3] = np.asarray(centre) + (rng.random((n, 3)) * 2.0 - 1.0) * half
    p[:, 3] = 1.0
    return p


def _crowded_dam_break():
    sc = scenes.dam_break()
    rng = np.random.default_rng(11)
    pos = np.concatenate([sc.positions, _blob(rng, (0.5, 0.5, 0.7), 0.075, 6000)])
    return sc, pos, None


def _crowded_coarse():
    sc = scenes.large(cell_rule="reference", counts=(40, 40, 20))
    assert sc.config.cell_size >= 2.0 * sc.config.smoothing_radius
    rng = np.random.default_rng(12)
    pos = np.concatenate([sc.positions, _blob(rng, (1.0, 1.0, 1.0), 0.02, 3000),
                          _blob(rng, (1.5, 1.5, 1.0), 0.0675, 4050)])
    return sc, pos, sc.collider_grid(0)


def _compare(sc, pos, col, order):
    from flowx_gb300.sph import Solver

    cfg = sc.config
    n = pos.shape[0]
    cfg.particle_count = n
    vel = np.zeros_like(pos)
    voxel = sc.collider_voxel if col is not None else 0.0
    ic = C.collider_binding(sc.collider_dims if col is not None else None, voxel)
    O.set_threads(O.max_threads())
    o = O.Oracle(C.push_constant_values(cfg, sc.dt, ic), pos, vel, collider=col, iterations=cfg.iterations)
    o.build_grid(0.0, order=order)
    o.substep(sc.dt, order=order)
    want = o.state()
    with Solver(cfg, pos, vel, collider=col, collider_voxel=voxel, exact=True,
                reference_order=order == O.ORDER_BITONIC) as s:
        s._build_grid(0.0)
        s._substep(sc.dt)
        for b in BUFS:
            np.testing.assert_array_equal(s.read(b), want[b], err_msg=b)
        # keys: the particles' entries (the bitonic network also reorders the
        # padding entries past them, key = cell count, which no pass reads)
        np.testing.assert_array_equal(s.read("keys", n), want["keys"][:n])
        np.testing.assert_array_equal(s.read("cell_start"), want["cell_start"])
        np.testing.assert_array_equal(s.read("cell_end"), want["cell_end"])
    return want


@pytest.mark.parametrize("order", [O.ORDER_STABLE, O.ORDER_BITONIC], ids=["cell_id", "reference"])
def test_crowded_cells_of_h_bit_exact_vs_oracle(order):
    sc, pos, col = _crowded_dam_break()
    want = _compare(sc, pos, col, order)
    cnt = np.where(want["cell_start"] >= 0, want["cell_end"] - want["cell_start"], 0)
    assert cnt.max() > 512  # a cell over MAX_CELL_SCAN took part


@pytest.mark.parametrize("order", [O.ORDER_STABLE, O.ORDER_BITONIC], ids=["cell_id", "reference"])
def test_crowded_coarse_cells_bit_exact_vs_oracle(order):
    sc, pos, col = _crowded_coarse()
    want = _compare(sc, pos, col, order)
    cnt = np.where(want["cell_start"] >= 0, want["cell_end"] - want["cell_start"], 0)
    assert cnt.max() > 512 and ((cnt > 120) & (cnt < 300)).any()
