"""Differentiable PBF substeps behind ``torch.autograd.Function``.

No reference counterpart: Flow-X's solver (solver/sph.py) is forward-only.
``AdjointSolver`` drives the library's checkpointed forward
(``flowx_adjoint_forward``: the substep of solver/sph.py:501-514 with the
reference's float32 expressions, particle arrays in id order) and its
hand-written adjoint (``flowx_substep_adjoint``). ``rollout`` makes the pair a
torch op: positions and velocities in, final splat grid and state out,
gradients flowing back to the initial positions and velocities. The
neighbour grid of each substep is held fixed in the adjoint.

PyTorch is used here for device buffers, streams and autograd only; all
forward and reverse arithmetic runs in the library's CUDA kernels.

``InverseProblem`` is the differentiable workload: the initial velocity is a
trilinear map of a 3x3x3 grid of 3-vectors spanning the domain, the loss the
squared L2 distance between the splat grid after the rollout and a target
splat produced by the same forward from a hidden control grid.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .config import SolverConfig, SurfaceConfig, collider_binding, push_constant_values, splat_push_values
from ._lib import FlowxError, Push


class AdjointSolver:
    """One scene's differentiable substeps on one GPU."""

    def __init__(self, config: SolverConfig, *, max_substeps: int, max_iterations: int | None = None,
                 surface: SurfaceConfig | None = None, collider=None, collider_voxel: float = 0.0,
                 device: int = 0):
        self.lib = _lib.load()
        self.config = config
        self.n = int(config.particle_count)
        self.surface = surface
        self.device = int(device)
        self.iterations = int(config.iterations)
        cfg = _lib.AdjointConfig()
        cfg.particle_count = self.n
        cfg.max_cells = int(config.cell_count)
        cfg.max_substeps = int(max_substeps)
        cfg.max_iterations = int(max_iterations or config.iterations)
        cfg.max_collider_voxels = int(np.asarray(collider).size) if collider is not None else 0
        cfg.max_surface_samples = int(surface.sample_count) if surface is not None else 0
        cfg.device = self.device
        self._h = ctypes.c_void_p()
        self._check(self.lib.flowx_adjoint_create(ctypes.byref(cfg), ctypes.byref(self._h)), None)
        self.collider_dims = None
        self.collider_voxel = 0.0
        if collider is not None and collider_voxel > 0.0:
            occ = np.asarray(collider)
            if occ.ndim != 3:
                raise ValueError("collider must be a (z, y, x) occupancy grid")
            if occ.dtype != np.uint8:
                occ = (occ > 0.5).astype(np.uint8)  # the reference's R32F > 0.5 test
            occ = np.ascontiguousarray(occ)
            dims = (ctypes.c_int32 * 3)(*occ.shape[::-1])
            self._check(self.lib.flowx_adjoint_set_collider(self._h, occ.ctypes.data, dims, float(collider_voxel)),
                        self._h)
            self.collider_dims = tuple(occ.shape[::-1])
            self.collider_voxel = float(collider_voxel)
        s = ctypes.c_void_p()
        self._check(self.lib.flowx_adjoint_get_stream(self._h, ctypes.byref(s)), self._h)
        self.stream = torch.cuda.ExternalStream(s.value, device=torch.device("cuda", self.device))
        self.token = 0
        self._dt = None

    def _check(self, rc, handle):
        if rc != _lib.FLOWX_OK:
            msg = self.lib.flowx_adjoint_last_error(handle)
            raise FlowxError(rc, msg.decode() if msg else "")

    def close(self):
        if self._h:
            self.lib.flowx_adjoint_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _push(self, dt):
        ic = collider_binding(self.collider_dims, self.collider_voxel)
        return Push.from_values(push_constant_values(self.config, dt, ic))

    def _splat_push(self, dt):
        ic = collider_binding(self.collider_dims, self.collider_voxel)
        return Push.from_values(splat_push_values(self.config, self.surface, dt, ic))

    def _tensor(self, x):
        t = torch.as_tensor(x, dtype=torch.float32, device=torch.device("cuda", self.device)).contiguous()
        if t.shape != (self.n, 4):
            raise ValueError(f"expected ({self.n}, 4) float32, got {tuple(t.shape)}")
        return t

    def forward(self, positions, velocities, substeps: int, dt: float):
        """Run ``substeps`` substeps; returns (surface or None, positions, velocities)."""
        pos = self._tensor(positions)
        vel = self._tensor(velocities)
        dev = torch.device("cuda", self.device)
        pos_out = torch.empty((self.n, 4), dtype=torch.float32, device=dev)
        vel_out = torch.empty_like(pos_out)
        surf = None
        splat = None
        if self.surface is not None:
            surf = torch.empty(self.surface.sample_count, dtype=torch.float32, device=dev)
            splat = ctypes.byref(self._splat_push(dt))
        torch.cuda.current_stream(dev).synchronize()
        rc = self.lib.flowx_adjoint_forward(self._h, ctypes.byref(self._push(dt)), self.iterations, int(substeps),
                                            pos.data_ptr(), vel.data_ptr(), pos_out.data_ptr(), vel_out.data_ptr(),
                                            splat, surf.data_ptr() if surf is not None else None)
        self._check(rc, self._h)
        self.stream.synchronize()
        self.token += 1
        self._dt = dt
        return surf, pos_out, vel_out

    def backward(self, surface_grad=None, positions_grad=None, velocities_grad=None):
        """Gradients of the initial (positions, velocities) for the last forward."""
        dev = torch.device("cuda", self.device)
        keep = []

        def ptr(t, shape):
            if t is None:
                return None
            t = torch.as_tensor(t, dtype=torch.float32, device=dev).contiguous().reshape(shape)
            keep.append(t)
            return t.data_ptr()

        gs = ptr(surface_grad, (-1,)) if self.surface is not None else None
        gp = ptr(positions_grad, (self.n, 4))
        gv = ptr(velocities_grad, (self.n, 4))
        out_p = torch.empty((self.n, 4), dtype=torch.float32, device=dev)
        out_v = torch.empty_like(out_p)
        torch.cuda.current_stream(dev).synchronize()
        rc = self.lib.flowx_substep_adjoint(self._h, gs, gp, gv, out_p.data_ptr(), out_v.data_ptr())
        self._check(rc, self._h)
        self.stream.synchronize()
        return out_p, out_v


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, velocities, solver, substeps, dt):
        surf, pos_out, vel_out = solver.forward(positions, velocities, substeps, dt)
        ctx.solver, ctx.substeps, ctx.dt, ctx.token = solver, substeps, dt, solver.token
        ctx.save_for_backward(positions, velocities)
        if surf is None:
            surf = torch.zeros(0, dtype=torch.float32, device=pos_out.device)
        return surf, pos_out, vel_out

    @staticmethod
    def backward(ctx, g_surface, g_pos, g_vel):
        solver = ctx.solver
        if solver.token != ctx.token:  # another forward ran since: record this one again
            positions, velocities = ctx.saved_tensors
            solver.forward(positions, velocities, ctx.substeps, ctx.dt)
        gp, gv = solver.backward(g_surface if solver.surface is not None else None, g_pos, g_vel)
        return gp, gv, None, None, None


def rollout(solver: AdjointSolver, positions: torch.Tensor, velocities: torch.Tensor, substeps: int, dt: float):
    """(surface, positions, velocities) after ``substeps`` substeps, differentiable
    with respect to ``positions`` and ``velocities`` (each (N, 4) float32 on the GPU)."""
    return _Rollout.apply(positions, velocities, solver, int(substeps), float(dt))


def trilinear_weights(positions: np.ndarray, lo, hi, nodes: int = 3):
    """(N, nodes^3) float32 weights of the trilinear map from a nodes^3 grid of
    control vectors spanning the box [lo, hi] (node index z, y, x) to particle
    positions: velocity = W @ control.reshape(nodes^3, 3)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    u = (positions[:, :3].astype(np.float64) - lo) / (hi - lo) * (nodes - 1)
    u = np.clip(u, 0.0, (nodes - 1) - 1e-9)
    i0 = np.floor(u).astype(np.int64)
    f = u - i0
    w = np.zeros((positions.shape[0], nodes**3))
    rows = np.arange(positions.shape[0])
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                wt = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (
                    f[:, 2] if dz else 1 - f[:, 2])
                node = ((i0[:, 2] + dz) * nodes + (i0[:, 1] + dy)) * nodes + (i0[:, 0] + dx)
                np.add.at(w, (rows, node), wt)
    return w.astype(np.float32)


class InverseProblem:
    """The differentiable workload: recover a hidden 3x3x3x3 control grid of
    initial velocities from the splat grid it produces after ``substeps``."""

    def __init__(self, scene, *, substeps=30, control_seed=4, hidden_seed=5, sigma_control=0.5, device=0):
        self.scene = scene
        self.substeps = int(substeps)
        self.dt = float(scene.dt)
        cfg = scene.config
        self.solver = AdjointSolver(cfg, max_substeps=self.substeps, surface=scene.surface, device=device)
        dev = torch.device("cuda", device)
        self.positions = torch.as_tensor(scene.positions, device=dev)
        self.weights = torch.as_tensor(trilinear_weights(scene.positions, cfg.lo, cfg.hi), device=dev)
        rng_h = np.random.default_rng(hidden_seed)
        rng_c = np.random.default_rng(control_seed)
        self.hidden = torch.as_tensor(rng_h.normal(0.0, sigma_control, (3, 3, 3, 3)).astype(np.float32), device=dev)
        self.initial = torch.as_tensor(rng_c.normal(0.0, sigma_control, (3, 3, 3, 3)).astype(np.float32), device=dev)
        with torch.no_grad():
            self.target = self.surface(self.hidden).detach().clone()

    def velocities(self, control: torch.Tensor) -> torch.Tensor:
        v3 = self.weights @ control.reshape(27, 3)
        return torch.cat([v3, torch.zeros_like(v3[:, :1])], dim=1)

    def surface(self, control: torch.Tensor) -> torch.Tensor:
        surf, _, _ = rollout(self.solver, self.positions, self.velocities(control), self.substeps, self.dt)
        return surf

    def loss(self, control: torch.Tensor, substeps: int | None = None) -> torch.Tensor:
        """Squared L2 distance of the splat after ``substeps`` (default: the
        problem's horizon) to the hidden control grid's splat at that horizon."""
        h = self.substeps if substeps is None else int(substeps)
        surf, _, _ = rollout(self.solver, self.positions, self.velocities(control), h, self.dt)
        d = surf - self.target_at(h)
        return (d * d).sum()

    def target_at(self, substeps: int) -> torch.Tensor:
        if substeps == self.substeps:
            return self.target
        cache = self.__dict__.setdefault("_targets", {})
        if substeps not in cache:
            with torch.no_grad():
                surf, _, _ = rollout(self.solver, self.positions, self.velocities(self.hidden), substeps, self.dt)
            cache[substeps] = surf.detach().clone()
        return cache[substeps]

    def horizon(self, step: int, steps: int, start: int = 3, reach: float = 0.75) -> int:
        """The continuation schedule: the horizon grows linearly from ``start``
        substeps to the full one over the first ``reach`` of the steps."""
        ramp = max(1, int(reach * steps))
        return min(self.substeps, start + (self.substeps - start) * step // ramp)

    def optimise(self, steps=200, lr=0.05, method="continuation"):
        """Adam on the control grid from the initial guess.

        method "adam": plain Adam on the full-horizon loss. Over 30 substeps
        that map is chaotic (the control gradient's norm is ~1e17, and a
        control change of 0.008 changes the loss by 15%), and plain Adam
        wanders upward.

        method "continuation": the horizon grows from 3 substeps to the full
        one over the first three quarters of the steps (``horizon``), each
        step's loss against the hidden grid's splat at that horizon; and every
        Adam step is kept only if it does not raise that loss, otherwise it is
        halved up to six times, and undone if it still does.

        Returns (losses at the full horizon before the first and after every
        step, final control).
        """
        control = self.initial.clone().requires_grad_(True)
        opt = torch.optim.Adam([control], lr=lr)
        with torch.no_grad():
            losses = [float(self.loss(control))]
        for step in range(int(steps)):
            h = self.substeps if method == "adam" else self.horizon(step, steps)
            opt.zero_grad()
            loss = self.loss(control, h)
            loss.backward()
            before = control.detach().clone()
            opt.step()
            if method == "continuation":
                with torch.no_grad():
                    trial = float(self.loss(control, h))
                    halvings = 0
                    while trial > float(loss) and halvings < 6:
                        control.copy_(before + 0.5 * (control - before))
                        trial = float(self.loss(control, h))
                        halvings += 1
                    if trial > float(loss):
                        control.copy_(before)
            elif method != "adam":
                raise ValueError(f"unknown method {method!r}")
            with torch.no_grad():
                losses.append(float(self.loss(control)))
        return losses, control.detach()
