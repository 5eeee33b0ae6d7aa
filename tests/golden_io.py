"""Loading helpers for the golden fixtures of tests/golden/."""

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TRACE_SCENES = ("dam_break", "dam_break_defaults", "pool_small", "pile")
STATE_BUFS = ("positions", "velocities", "lambda", "predicted", "delta", "normal", "keys", "cell_start", "cell_end")


class Trace:
    def __init__(self, name):
        self.name = name
        self.z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
        self.meta = json.loads(bytes(self.z["meta"]).decode())
        self.push = {k: tuple(v) for k, v in self.meta["push"].items()}
        self.collider = self.z["collider"] if "collider" in self.z.files else None

    def init_state(self):
        return {b: self.z[f"init_{b}"].copy() for b in STATE_BUFS}

    def passes(self):
        """[(index, pass_name, {buf: array})] in dispatch order."""
        out = []
        for i, name in enumerate(self.meta["order"]):
            prefix = f"p{i:02d}_{name}_"
            bufs = {k[len(prefix):]: self.z[k] for k in self.z.files if k.startswith(prefix)}
            out.append((i, name, bufs))
        return out

    def substep_state(self, k):
        return {b: self.z[f"sub{k:02d}_{b}"] for b in ("positions", "velocities", "lambda", "predicted")}


def membership(keys, cell_start, cell_end):
    """{cell: sorted ids} from a key array and cell ranges."""
    out = {}
    for c in np.nonzero(cell_start >= 0)[0]:
        s, e = int(cell_start[c]), int(cell_end[c])
        out[int(c)] = sorted(int(v) for v in keys[s:e, 1])
    return out


def assert_close(name, got, want, rel=1e-5, abs_floor=1e-30):
    """Per-element |got - want| <= rel * max(|want|) (a scale-aware bound for a
    float32 pass output computed with a different summation order or
    rounding of constants)."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    assert np.isfinite(got).all() == np.isfinite(want).all(), name
    scale = max(float(np.abs(want).max()) if want.size else 0.0, abs_floor)
    err = float(np.abs(got - want).max()) if want.size else 0.0
    assert err <= rel * scale, f"{name}: max err {err:.3e} > {rel:.1e} * {scale:.3e}"
    return err / scale
