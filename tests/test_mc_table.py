"""The library's marching-cubes case table (derived at set-up, no GPU) equals
the reference's derived TRI_TABLE (solver/marching_cubes.py:122-164), stored
in tests/golden/mc_golden.npz by make_mc_golden.py."""

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_case_table_equals_reference():
    from flowx_gb300 import build
    from flowx_gb300.surface import case_table

    build.build()
    z = np.load(os.path.join(HERE, "golden", "mc_golden.npz"))
    table, counts = case_table()
    np.testing.assert_array_equal(counts, z["tri_count"])
    np.testing.assert_array_equal(table, z["tri_table"])
    assert counts[0] == 0 and counts[255] == 0 and counts.max() <= 5
