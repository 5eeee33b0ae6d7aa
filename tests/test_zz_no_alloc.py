"""flowx_build_grid_static (the grid build that allocates nothing, scratch in
a static device array) against flowx_build_grid on the same predicted
positions: keys and cell ranges are integer work, compared exactly, over
consecutive calls that reuse the static scratch.

The file name sorts last so that the suite also runs it after every other
GPU test in the same process."""

import ctypes

import numpy as np
import pytest

from flowx_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 65536
MAX_CELLS = 262144
ERR_ARG = 1  # FLOWX_ERR_ARG
ERR_CAPACITY = 4  # FLOWX_ERR_CAPACITY


def _static_build(predicted_id_order, push, key_count, cells):
    """One flowx_build_grid_static call on device buffers owned by the caller."""
    import torch

    lib = _lib.load()
    n = int(predicted_id_order.shape[0])
    pred = torch.from_numpy(np.ascontiguousarray(predicted_id_order, np.float32)).to("cuda:0")
    keys = torch.full((key_count, 4), 7.0, dtype=torch.float32, device="cuda:0")
    start = torch.full((cells,), 7.0, dtype=torch.float32, device="cuda:0")
    end = torch.full((cells,), 7.0, dtype=torch.float32, device="cuda:0")
    stream = torch.cuda.current_stream(0)
    rc = lib.flowx_build_grid_static(pred.data_ptr() if n else None, n, ctypes.byref(push), keys.data_ptr(),
                                     key_count, start.data_ptr(), end.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.FLOWX_OK, lib.flowx_build_grid_static_error().decode()
    torch.cuda.synchronize(0)
    return keys.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy()


def _context_build(solver, predicted_id_order):
    solver.write("predicted", predicted_id_order)
    solver._build_grid(0.0)
    return solver.read("keys"), solver.read("cell_start"), solver.read("cell_end")


def _assert_same(got, want):
    for g, w, name in zip(got, want, ("keys", "cell_start", "cell_end")):
        assert g.shape == w.shape, name
        assert np.array_equal(g, w), f"{name}: {np.count_nonzero(g != w)} entries differ"


def _clustered(n, cfg, seed):
    """Half the particles packed into a few cells (more than 32 per cell, the
    per-cell network limit), the rest spread over and past the domain."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(cfg.lo, np.float32), np.asarray(cfg.hi, np.float32)
    out = np.ones((n, 4), np.float32)
    half = n // 2
    centres = lo + (hi - lo) * rng.random((4, 3), dtype=np.float32)
    out[:half, :3] = centres[rng.integers(0, 4, half)] + 1e-3 * rng.standard_normal((half, 3)).astype(np.float32)
    span = hi - lo
    out[half:, :3] = lo - 0.1 * span + 1.2 * span * rng.random((n - half, 3), dtype=np.float32)
    return out


def test_static_grid_matches_build_grid_on_consecutive_calls():
    from flowx_gb300.sph import Solver

    sc = scenes.inverse_problem()
    cfg = sc.config
    assert sc.n <= MAX_PARTICLES and cfg.cell_count <= MAX_CELLS
    with Solver(cfg, sc.positions, sc.velocities, exact=True) as s:
        push = s.push(0.0)
        # Call 1: the seeded lattice.
        want = _context_build(s, sc.positions)
        _assert_same(_static_build(sc.positions, push, cfg.sorted_count, cfg.cell_count), want)
        # Call 2: predicted positions after two substeps.
        dt = sc.dt
        s._substep(dt)
        s._substep(dt)
        pred = s.read("predicted")
        want = _context_build(s, pred)
        _assert_same(_static_build(pred, push, cfg.sorted_count, cfg.cell_count), want)
        # Call 3: crowded cells (the block-per-cell sort) and out-of-box particles.
        crowd = _clustered(sc.n, cfg, seed=11)
        want = _context_build(s, crowd)
        got = _static_build(crowd, push, cfg.sorted_count, cfg.cell_count)
        _assert_same(got, want)
        counts = np.where(want[1] >= 0, want[2] - want[1], 0)
        assert counts.max() > 32 and counts.sum() == sc.n


def test_static_grid_small_scene_and_reuse_after_larger_call():
    """A smaller grid right after a larger one: stale counters or offsets
    from the previous call must not leak into this one."""
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    cfg = sc.config
    with Solver(cfg, sc.positions, sc.velocities, exact=True) as s:
        push = s.push(0.0)
        for seed in (1, 2):
            pts = _clustered(sc.n, cfg, seed)
            want = _context_build(s, pts)
            _assert_same(_static_build(pts, push, cfg.sorted_count, cfg.cell_count), want)


def test_static_grid_allocates_nothing_after_the_first_call():
    """The first call on a device is a warm-up (the runtime may load the
    library's module there, reserving the static scratch); the calls after
    it leave the device's free memory unchanged. The caller's buffers are
    made once, before the calls."""
    import torch

    from flowx_gb300.sph import Solver

    lib = _lib.load()
    sc = scenes.dam_break()
    cfg = sc.config
    with Solver(cfg, sc.positions, sc.velocities) as s:
        push = s.push(0.0)
    pred = torch.from_numpy(np.ascontiguousarray(sc.positions, np.float32)).to("cuda:0")
    keys = torch.zeros((cfg.sorted_count, 4), dtype=torch.float32, device="cuda:0")
    start = torch.zeros(cfg.cell_count, dtype=torch.float32, device="cuda:0")
    end = torch.zeros(cfg.cell_count, dtype=torch.float32, device="cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream(0).cuda_stream)

    def call():
        rc = lib.flowx_build_grid_static(pred.data_ptr(), sc.n, ctypes.byref(push), keys.data_ptr(),
                                         cfg.sorted_count, start.data_ptr(), end.data_ptr(), stream)
        assert rc == _lib.FLOWX_OK, lib.flowx_build_grid_static_error().decode()
        torch.cuda.synchronize(0)
        return torch.cuda.mem_get_info(0)[0]

    before = call()  # warm-up; free memory after it
    free = [call() for _ in range(3)]
    assert all(f == before for f in free), (before, free)
    first = (keys.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy())
    call()
    _assert_same((keys.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy()), first)


def test_static_grid_rejects_sizes_beyond_the_static_scratch():
    import torch

    lib = _lib.load()
    sc = scenes.dam_break()
    from flowx_gb300.sph import Solver

    with Solver(sc.config, sc.positions, sc.velocities) as s:
        push = s.push(0.0)
    buf = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    p = buf.data_ptr()
    big = _lib.Push.from_buffer_copy(bytes(push))
    big.i_layout[0] = MAX_PARTICLES + 1
    rc = lib.flowx_build_grid_static(p, MAX_PARTICLES + 1, ctypes.byref(big), p, MAX_PARTICLES + 1, p, p, None)
    assert rc == ERR_CAPACITY
    assert b"65536" in lib.flowx_build_grid_static_error()
    wide = _lib.Push.from_buffer_copy(bytes(push))
    wide.i_layout[0] = 1
    wide.i_grid[0], wide.i_grid[1], wide.i_grid[2] = 128, 64, 33
    wide.i_grid[3] = 128 * 64 * 33
    rc = lib.flowx_build_grid_static(p, 1, ctypes.byref(wide), p, 1, p, p, None)
    assert rc == ERR_CAPACITY
    assert b"262144" in lib.flowx_build_grid_static_error()
    rc = lib.flowx_build_grid_static(p, 2, ctypes.byref(big), p, 1, p, p, None)
    assert rc == ERR_ARG
