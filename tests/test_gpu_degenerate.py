"""Degenerate states stay bounded: 10,000 particles at one point fill one cell
far above the block sorter's limit (4,096). The grid still has its key
column sorted by cell, ids forming a permutation and exact cell ranges (the
order inside that cell is the scatter's, as the reference's unstable bitonic
sort leaves it arbitrary), and a substep completes with finite positions."""

import numpy as np
import pytest

from flowx_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_one_crowded_cell_builds_and_steps():
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    cfg = sc.config
    n = 10000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (0.45, 0.45, 0.45)
    pos[:, 3] = 1.0
    with Solver(cfg, pos, np.zeros_like(pos)) as s:
        s._build_grid(0.0)
        keys = s.read("keys")
        cs, ce = s.read("cell_start"), s.read("cell_end")
        real = keys[:n]
        assert (np.diff(real[:, 0]) >= 0).all()
        assert np.array_equal(np.sort(real[:, 1].astype(np.int64)), np.arange(n))
        cell = int(real[0, 0])
        assert (real[:, 0] == cell).all() and cs[cell] == 0 and ce[cell] == n
        assert (np.delete(cs, cell) == -1).all()
        s._substep(sc.dt)
        assert np.isfinite(s.read("positions")).all()
