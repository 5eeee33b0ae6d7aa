"""The float64 torch re-expression (oracle/adjoint64.py) that checks the
library's adjoint is itself checked here, on the CPU:

* its forward equals oracle/ref64.py's float64 passes (the restatement of
  the reference's GLSL passes) over several substeps, with cohesion, a
  collider and the splat;
* its torch-autograd gradient equals float64 central differences (eps 1e-4)
  along random directions.
"""

import numpy as np
import pytest
import torch

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import adjoint64 as A
from oracle import ref64 as R


def _scene(name):
    if name == "pool":
        sc = scenes.pool(counts=(24, 12, 8), extent=1.0)
        return sc, sc.collider_grid(0), sc.collider_voxel
    return scenes.inverse_problem(n_block=(20, 10, 10)), None, 0.0


def _ref64_rollout(sc, prm, vel0, substeps, surface):
    n = sc.n
    pos = np.c_[sc.positions[:, :3].astype(np.float64), np.ones(n)]
    st = {"positions": pos, "velocities": np.c_[vel0, np.zeros(n)], "predicted": pos.copy(),
          "lambda": np.zeros((n, 4)), "delta": np.zeros((n, 4)), "normal": np.zeros((n, 4))}
    st["keys"], st["cell_start"], st["cell_end"] = R.build_grid(st["predicted"], prm, sc.config.sorted_count)
    for _ in range(substeps):
        st = R.substep(st, prm, sc.config.sorted_count, sc.config.iterations)
    surf = R.splat(st, prm, dims=surface.dims, spacing=surface.spacing, kernel_radius=surface.kernel_radius,
                   surface_lo=surface.lo)
    return st, surf


@pytest.mark.parametrize("name", ["block", "pool"])
def test_torch_forward_equals_ref64(name):
    sc, col, voxel = _scene(name)
    prm = A.params(sc.config, sc.dt, col, voxel)
    surface = C.surface_for_dims(sc.config, 24)
    vel0 = np.random.default_rng(1).normal(0.0, 0.5, (sc.n, 3))
    st, surf = _ref64_rollout(sc, prm, vel0, 2, surface)
    tsurf, tst = A.rollout(torch.tensor(sc.positions[:, :3], dtype=torch.float64), torch.tensor(vel0), prm,
                           sc.config.sorted_count, sc.config.iterations, 2, surface)
    scale = np.abs(st["positions"][:, :3]).max()
    assert np.abs(tst["positions"].numpy() - st["positions"][:, :3]).max() <= 1e-12 * scale
    assert np.abs(tst["velocities"].numpy() - st["velocities"][:, :3]).max() <= 1e-9
    assert np.abs(tsurf.numpy() - surf).max() <= 1e-9 * max(np.abs(surf).max(), 1.0)


@pytest.mark.parametrize("name", ["block", "pool"])
def test_torch_autograd_equals_central_differences(name):
    sc, col, voxel = _scene(name)
    prm = A.params(sc.config, sc.dt, col, voxel)
    surface = C.surface_for_dims(sc.config, 24)
    rng = np.random.default_rng(2)
    vel0 = torch.tensor(rng.normal(0.0, 0.5, (sc.n, 3)))
    pos0 = torch.tensor(sc.positions[:, :3], dtype=torch.float64)
    ws = torch.tensor(rng.normal(size=surface.sample_count))
    wp = torch.tensor(rng.normal(size=(sc.n, 3)))

    def loss(v):
        surf, st = A.rollout(pos0, v, prm, sc.config.sorted_count, sc.config.iterations, 2, surface)
        return (surf * ws).sum() + (st["positions"] * wp).sum() + 0.1 * (st["velocities"] ** 2).sum()

    v = vel0.clone().requires_grad_(True)
    loss(v).backward()
    for _ in range(2):
        u = torch.tensor(rng.normal(size=(sc.n, 3)))
        fd = A.central_difference(loss, vel0, u, eps=1e-4)
        ad = float((v.grad * u).sum())
        assert abs(ad - fd) <= 1e-5 * abs(fd), (ad, fd)
