"""The oracle's marching cubes (oracle/mc.py) against the reference's own
table and meshes (solver/marching_cubes.py, stored in
tests/golden/mc_golden.npz by make_mc_golden.py): identical case table,
identical vertices (float64 bits) and triangles. The GPU extraction is then
checked against this oracle at sizes the fixtures do not hold."""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    return np.load(os.path.join(HERE, "golden", "mc_golden.npz"))


def test_case_table_equals_reference():
    from oracle import mc

    z = _golden()
    table, counts = mc.case_table()
    np.testing.assert_array_equal(counts, z["tri_count"])
    np.testing.assert_array_equal(table, z["tri_table"])


@pytest.mark.parametrize("name", ("sphere", "noise", "splat", "empty"))
def test_extract_equals_reference(name):
    from oracle import mc

    z = _golden()
    lat = z[f"{name}_lattice"]
    dims = tuple(int(v) for v in lat[:3])
    verts, tris = mc.extract(z[f"{name}_field"], dims, tuple(lat[3:6]), float(lat[6]), float(lat[7]))
    np.testing.assert_array_equal(tris, z[f"{name}_triangles"])
    np.testing.assert_array_equal(verts, z[f"{name}_vertices"])


def test_degenerate_lattices():
    from oracle import mc

    for dims in ((1, 4, 4), (4, 1, 4), (4, 4, 1)):
        v, t = mc.extract(np.ones(int(np.prod(dims)), np.float32), dims, (0, 0, 0), 1.0, 0.5)
        assert v.shape == (0, 3) and t.shape == (0, 3)
    # all inside: no surface
    v, t = mc.extract(np.ones(64, np.float32), (4, 4, 4), (0, 0, 0), 1.0, 0.5)
    assert v.shape == (0, 3) and t.shape == (0, 3)
