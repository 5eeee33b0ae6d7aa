"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

* Pass by pass against the golden traces of the reference's own GLSL passes:
  every pass runs on exactly the inputs the reference's pass saw (uploaded,
  including the reference's bitonic key order, so neighbour sums run in the
  reference's order), and its outputs are compared with the reference's
  (bit-exact, except delta's pow(ratio, 4.0), which the reference's harness
  takes from glibc's powf: within 1e-6 of the buffer's scale) and with the C
  oracle on the same inputs (bit-exact: same float32 operations in the same
  order, no FMA contraction on either side).
* Whole fused substeps against the oracle in the (cell, id) order the CUDA
  grid build emits: bit-exact over several substeps, graph and non-graph.
"""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from golden_io import TRACE_SCENES, Trace, assert_close, membership
from oracle import oracle as O
from rounding import assert_within_sensitivity, per_particle, perturbed_state, ulp_neighbour

pytestmark = pytest.mark.gpu

PARTICLE_BUFS = ("positions", "velocities", "lambda", "predicted", "delta", "normal")


def _solver(tr, **kw):
    from flowx_gb300.sph import Solver

    cfg = C.config_from_push(tr.push)
    cfg.iterations = tr.meta["iterations"]
    z = tr.z
    voxel = tr.meta.get("collider_voxel", 0.0)
    return Solver(cfg, z["init_positions"], z["init_velocities"], collider=tr.collider, collider_voxel=voxel,
                  max_cells=tr.meta["c"], **kw)


def _load_state(s, state):
    for b in PARTICLE_BUFS:
        if b in state:
            s.write(b, state[b])
    if "keys" in state:
        s.write("keys", state["keys"])
        for b in ("cell_start", "cell_end"):
            if b in state:
                s.write(b, state[b])


@pytest.mark.parametrize("scene", TRACE_SCENES)
def test_passes_match_reference_and_oracle(scene):
    tr = Trace(scene)
    dt = tr.meta["dt"]
    state = tr.init_state()
    o = O.Oracle(tr.push, state["positions"], state["velocities"], collider=tr.collider,
                 iterations=tr.meta["iterations"])
    pass_ids = {"normal": O.NORMAL, "predict": O.PREDICT, "lambda": O.LAMBDA, "delta": O.DELTA,
                "apply_delta": O.APPLY_DELTA, "velocity": O.VELOCITY, "xsph": O.XSPH, "finalize": O.FINALIZE}
    with _solver(tr) as s:
        _load_state(s, state)
        for idx, name, outs in tr.passes():
            tag = f"{scene} pass {idx} {name}"
            if name == "build_grid":
                s._build_grid(dt)
                keys = s.read("keys", tr.meta["s"])
                cs, ce = s.read("cell_start"), s.read("cell_end")
                np.testing.assert_array_equal(keys[:, 0], outs["keys"][:, 0], err_msg=tag)
                np.testing.assert_array_equal(cs, outs["cell_start"], err_msg=tag)
                np.testing.assert_array_equal(ce, outs["cell_end"], err_msg=tag)
                assert membership(keys, cs, ce) == membership(outs["keys"], outs["cell_start"], outs["cell_end"])
                # continue in the reference's own slot order
                s.write("keys", outs["keys"])
            else:
                o.load(state)
                o.run_pass(pass_ids[name], o.push(dt))
                s.run_pass(name, dt)
                for b, want in outs.items():
                    got = s.read(b)
                    oracle_out = getattr(o, "lambda_" if b == "lambda" else b)
                    np.testing.assert_array_equal(got, oracle_out, err_msg=f"{tag}.{b} vs oracle")
                    if name == "delta":
                        assert_close(f"{tag}.{b} vs reference", got, want, rel=1e-6)
                    else:
                        np.testing.assert_array_equal(got, want, err_msg=f"{tag}.{b} vs reference")
            state.update({k: v.copy() for k, v in outs.items()})
            _load_state(s, outs)


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile", "dam_break_defaults"])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("passes", ["thread", "warp"])
def test_fused_substeps_bit_exact_vs_oracle(scene, graph, passes):
    """EXACT fused substeps against the oracle, with the neighbour passes one
    thread per particle and one warp per particle (pbf_warp.cu)."""
    tr = Trace(scene)
    dt = tr.meta["dt"]
    iters = tr.meta["iterations"]
    z = tr.z
    o = O.Oracle(tr.push, z["init_positions"], z["init_velocities"], collider=tr.collider, iterations=iters)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    nsub = 3
    with _solver(tr, exact=True, passes=passes) as s:
        s._build_grid(0.0)
        if graph:
            s.step_substeps(dt, nsub)
        else:
            for _ in range(nsub):
                s._substep(dt)
        for _ in range(nsub):
            o.substep(dt, order=O.ORDER_STABLE)
        want = o.state()
        for b in ("positions", "velocities", "predicted", "lambda", "normal"):
            np.testing.assert_array_equal(s.read(b), want[b], err_msg=f"{scene} {b}")
        np.testing.assert_array_equal(s.read("keys", tr.meta["s"]), want["keys"])
        np.testing.assert_array_equal(s.read("cell_start"), want["cell_start"])
        np.testing.assert_array_equal(s.read("cell_end"), want["cell_end"])


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile", "dam_break_defaults"])
def test_fast_warp_and_thread_passes_are_bit_identical(scene):
    """FAST substeps (a frame, graph-launched, with the fused normal pass) give
    the same bits whether the neighbour passes run one warp or one thread per
    particle: the warp kernels fold the same terms in the same order."""
    tr = Trace(scene)
    out = {}
    for passes in ("thread", "warp"):
        with _solver(tr, exact=False, passes=passes) as s:
            s._build_grid(0.0)
            s.step_substeps(tr.meta["dt"], 4)
            out[passes] = {b: s.read(b) for b in ("positions", "velocities", "predicted", "lambda", "normal")}
    for b in out["thread"]:
        np.testing.assert_array_equal(out["warp"][b], out["thread"][b], err_msg=f"{scene} {b}")


@pytest.mark.parametrize("scene", ["dam_break", "pool_small"])
def test_fused_substeps_across_calls_bit_exact(scene):
    """Substeps split over several calls (a graph, a single substep, then an
    upload of moved predicted positions and another graph): the normal pass
    reuses the previous XSPH pass's row masks only while nothing has changed
    positions or the grid, and stays bit-exact against the oracle."""
    tr = Trace(scene)
    dt = tr.meta["dt"]
    iters = tr.meta["iterations"]
    z = tr.z
    o = O.Oracle(tr.push, z["init_positions"], z["init_velocities"], collider=tr.collider, iterations=iters)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    with _solver(tr, exact=True) as s:
        s._build_grid(0.0)
        s.step_substeps(dt, 2)
        s._substep(dt)
        for _ in range(3):
            o.substep(dt, order=O.ORDER_STABLE)
        moved = o.state()["predicted"].copy()
        moved[:, :3] += np.random.default_rng(5).uniform(-1e-4, 1e-4, (moved.shape[0], 3)).astype(np.float32)
        s.write("predicted", moved)
        o.predicted[...] = moved
        s.step_substeps(dt, 2)
        for _ in range(2):
            o.substep(dt, order=O.ORDER_STABLE)
        want = o.state()
        for b in ("positions", "velocities", "predicted", "lambda", "normal"):
            np.testing.assert_array_equal(s.read(b), want[b], err_msg=f"{scene} {b}")


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile"])
@pytest.mark.parametrize("graph", [False, True])
def test_reference_order_substeps_match_reference(scene, graph):
    """The reference's own grid order (FLOWX_FLAG_REFERENCE_ORDER: its bitonic
    network, run on the GPU) with its expressions (EXACT), from the seeded
    state through every substep the trace holds, cohesion on: bit-exact
    against the oracle running the same network after every substep (every
    buffer, keys with ids), and within 1e-5 h of the reference's own passes
    after the first (measured 6e-7 to 1.2e-6 h: delta's pow ulp is all that
    differs). The seeded substeps amplify that ulp (a 1-ulp change of the
    input positions moves the result by ~2e-4 h, tests/rounding.py), so the
    distance to the reference after later substeps is reported, not bounded."""
    tr = Trace(scene)
    h = tr.push["f_sph"][0]
    dt = tr.meta["dt"]
    z = tr.z
    o = O.Oracle(tr.push, z["init_positions"], z["init_velocities"], collider=tr.collider,
                 iterations=tr.meta["iterations"])
    o.build_grid(0.0, order=O.ORDER_BITONIC)
    with _solver(tr, exact=True, reference_order=True) as s:
        s._build_grid(0.0)
        n = tr.meta["n"]
        np.testing.assert_array_equal(s.read("keys", n), o.keys[:n], err_msg=f"{scene} seed grid")
        for k in range(1, tr.meta["substeps"] + 1):
            if graph:
                s.step_substeps(dt, 1)
            else:
                s._substep(dt)
            o.substep(dt, order=O.ORDER_BITONIC)
            want = o.state()
            # keys: the particles' entries (the padding entries past them hold
            # key = cell count, which no pass reads: sph_cell_range.glsl:19-21)
            for b in ("positions", "velocities", "predicted", "lambda", "normal", "keys", "cell_start",
                      "cell_end"):
                got = s.read(b, n if b == "keys" else None)
                exp = want[b][:n] if b == "keys" else want[b]
                np.testing.assert_array_equal(got, exp, err_msg=f"{scene} substep {k} {b} vs oracle")
            ref = tr.substep_state(k)["positions"]
            err = np.abs(s.read("positions")[:, :3].astype(np.float64) - ref[:, :3]).max()
            print(f"{scene} reference order, substep {k}: {err / h:.2e} h from the reference")
            if k == 1:
                assert err <= 1e-5 * h, (k, err / h)


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile"])
def test_first_substep_within_tolerance_of_reference(scene):
    """One substep from the seeded state, cohesion on, against the reference's
    own passes, in the GPU's (cell, id) grid order. The visiting order inside
    a cell differs from the reference's bitonic one, and the cohesion term
    amplifies the resulting roundings (its normals cancel for interior
    particles and enter the predict step through 1/|n|): both arithmetic
    modes stay within 2e-4 h, EXACT measured at 2-9e-5 h."""
    tr = Trace(scene)
    h = tr.push["f_sph"][0]
    for exact in (True, False):
        with _solver(tr, exact=exact) as s:
            s._build_grid(0.0)
            s._substep(tr.meta["dt"])
            got = s.read("positions")
        want = tr.substep_state(1)["positions"]
        err = np.abs(got[:, :3].astype(np.float64) - want[:, :3]).max()
        print(f"{scene} {'EXACT' if exact else 'FAST'} (cell, id) order vs reference: {err / h:.2e} h")
        assert err <= 2e-4 * h, (exact, err / h)


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile"])
def test_splat_matches_reference_and_oracle(scene):
    tr = Trace(scene)
    sp = {k: tuple(v) for k, v in tr.meta["splat_push"].items()}
    dims = sp["i_surface"][:3]
    samples = int(np.prod(dims))
    final = tr.substep_state(tr.meta["substeps"])
    with _solver(tr, max_surface_samples=samples) as s:
        _load_state(s, {"positions": final["positions"], "keys": tr.z["last_keys"],
                        "cell_start": tr.z["last_cell_start"], "cell_end": tr.z["last_cell_end"]})
        import ctypes
        from flowx_gb300 import _lib

        out = np.empty(samples, np.float32)
        push = _lib.Push.from_values(sp)
        _lib.check(s.lib.flowx_splat(s.ctx, ctypes.byref(push), out.ctypes.data, out.nbytes), s.ctx)
    o = O.Oracle(tr.push, final["positions"], final["velocities"], collider=tr.collider)
    o.load({"keys": tr.z["last_keys"], "cell_start": tr.z["last_cell_start"], "cell_end": tr.z["last_cell_end"]})
    np.testing.assert_array_equal(out, o.splat(sp))
    assert_close(f"{scene} splat vs reference", out, tr.z["splat"], rel=1e-5)


def test_dam_break_density_holds_near_rest():
    """The reference's only physics assertion (scripts/smoke_test.py:107-134):
    mean density within 15% of rest after 3 frames."""
    from flowx_gb300.sph import Solver

    scene = scenes.dam_break()
    cfg = scene.config
    with Solver(cfg, scene.positions, scene.velocities) as s:
        s._build_grid(0.0)
        for _ in range(3):
            s.step_substeps(scene.dt, scene.substeps_per_frame)
        rho = s.read("lambda")[:, 0]
        pos = s.read("positions")
    assert np.isfinite(pos).all()
    err = abs(rho.mean() - cfg.rest_density) / cfg.rest_density
    assert err < 0.15, err


def _stable_no_cohesion_scene():
    """dam_break geometry without the cohesion term: a well-conditioned
    substep, where float32 evaluations differing in rounding stay within
    1e-5 h of each other after one substep."""
    scene = scenes.dam_break()
    scene.config.surface_tension = 0.0
    return scene


def _oracle_first_substep(tr, positions):
    z = tr.z
    o = O.Oracle(tr.push, positions, z["init_velocities"], collider=tr.collider, iterations=tr.meta["iterations"])
    o.build_grid(0.0, order=O.ORDER_STABLE)
    o.substep(tr.meta["dt"], order=O.ORDER_STABLE)
    return o.positions.copy()


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile"])
def test_fast_first_substep_within_rounding_sensitivity_of_oracle(scene):
    """The benchmarked arithmetic (FAST), cohesion on, one substep from the
    seeded lattice against the oracle in the same grid order. That substep is
    ill-conditioned (tests/rounding.py): a 1-ulp change of the input
    positions moves the oracle's own result by up to ~2e-4 h. FAST stays
    within a small factor of that at every quantile."""
    tr = Trace(scene)
    h = tr.push["f_sph"][0]
    want = _oracle_first_substep(tr, tr.z["init_positions"])
    noise = per_particle(_oracle_first_substep(tr, ulp_neighbour(tr.z["init_positions"])), want, h)
    with _solver(tr, exact=False) as s:
        s._build_grid(0.0)
        s.step_substeps(tr.meta["dt"], 1)
        got = s.read("positions")
    assert_within_sensitivity(f"{scene} seeded", per_particle(got, want, h), noise)


def test_fast_substep_within_1e5h_of_oracle_when_well_conditioned():
    """The dam break after 8 frames (the oracle's own run, cohesion on): there
    a 1-ulp change of the input positions moves one substep's result by
    under 4e-6 h for 99% of the particles (1.8e-5 h at most), and FAST must
    stay within 1e-5 h of the oracle in every particle position."""
    from flowx_gb300.sph import Solver

    scene = scenes.dam_break()
    cfg = scene.config
    h = cfg.smoothing_radius
    push = C.push_constant_values(cfg, scene.dt)
    o = O.Oracle(push, scene.positions, scene.velocities, iterations=cfg.iterations)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    for _ in range(8 * scene.substeps_per_frame):
        o.substep(scene.dt, order=O.ORDER_STABLE)
    st = o.state()

    def oracle_one(state):
        q = O.Oracle(push, state["positions"], state["velocities"], iterations=cfg.iterations)
        q.predicted[...] = state["predicted"]
        q.lambda_[...] = state["lambda"]
        q.build_grid(0.0, order=O.ORDER_STABLE)
        q.substep(scene.dt, order=O.ORDER_STABLE)
        return q.positions.copy()

    want = oracle_one(st)
    noise = per_particle(oracle_one(perturbed_state(st)), want, h)
    with Solver(cfg, st["positions"], st["velocities"]) as s:
        s.write("predicted", st["predicted"])
        s.write("lambda", st["lambda"])
        s._build_grid(0.0)
        s.step_substeps(scene.dt, 1)
        got = s.read("positions")
    err = per_particle(got, want, h)
    print(f"dam break after 8 frames: FAST max {err.max():.2e} h, oracle 1-ulp sensitivity max {noise.max():.2e} h, "
          f"99% {np.quantile(noise, 0.99):.2e} h")
    assert np.quantile(noise, 0.99) <= 1e-5 / 2
    assert err.max() <= 1e-5, err.max()


def test_fast_substep_within_1e5h_of_oracle():
    from flowx_gb300.sph import Solver

    scene = _stable_no_cohesion_scene()
    cfg = scene.config
    with Solver(cfg, scene.positions, scene.velocities) as s:
        s._build_grid(0.0)
        s._substep(scene.dt)
        got = {b: s.read(b) for b in ("positions", "velocities", "lambda")}
    o = O.Oracle(C.push_constant_values(cfg, scene.dt), scene.positions, scene.velocities, iterations=cfg.iterations)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    o.substep(scene.dt, order=O.ORDER_STABLE)
    err = np.abs(got["positions"][:, :3].astype(np.float64) - o.positions[:, :3]).max()
    assert err <= 1e-5 * cfg.smoothing_radius, err / cfg.smoothing_radius
    assert_close("fast lambda", got["lambda"], o.lambda_, rel=1e-4)


@pytest.mark.parametrize("scene", ["dam_break", "pool_small", "pile"])
def test_fast_passes_track_exact(scene):
    """FAST and EXACT fused substeps stay together over a frame (4 substeps)
    up to float32 rounding amplified by the dynamics."""
    tr = Trace(scene)
    h = tr.push["f_sph"][0]
    out = {}
    for exact in (True, False):
        with _solver(tr, exact=exact) as s:
            s._build_grid(0.0)
            s.step_substeps(tr.meta["dt"], 1)
            out[exact] = s.read("positions")
    err = np.abs(out[True][:, :3].astype(np.float64) - out[False][:, :3]).max()
    assert err <= 1e-4 * h, err / h
