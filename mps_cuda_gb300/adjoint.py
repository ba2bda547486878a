"""Differentiable DFSPH rollouts.

`AdjointRollout` drives the adjoint C ABI (mps_adjoint_forward / mps_adjoint_backward): a forward
of `nsteps` steps with a checkpoint every `every` steps, then the reverse sweep that recomputes
each segment from its checkpoint (neighbour lists rebuilt) and runs the hand-written adjoint
kernels step by step.  `rollout` wraps it in a torch.autograd.Function so that any torch loss of
the final state back-propagates to the initial positions and velocities and to the viscosity and
surface-tension coefficients.  `com_loss` is the loss of the adjoint benchmark: per scene, the
squared distance of the final fluid centre of mass to a target plus w times the mean squared
final speed.

The simulation must use fixed solver iterations (fixed_iters > 0) and the Jacobi
viscosity / surface-tension solve (visc_solver = VISC_JACOBI).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class AdjointRollout:
    """Forward + reverse of `nsteps` steps on a Simulation or BatchedSimulation."""

    def __init__(self, sim, nsteps: int, every: int = 20):
        self.sim = sim
        self.nsteps = int(nsteps)
        self.every = int(every)
        self.lib = sim.lib

    def memory_bytes(self) -> int:
        return int(self.lib.mps_adjoint_memory(self.sim.h, self.nsteps, self.every))

    def reserve(self) -> None:
        """Allocates the checkpoint and tape buffers now (else on the first forward)."""
        L.check(self.lib.mps_adjoint_reserve(self.sim.h, self.nsteps, self.every))

    def forward(self, pos4: np.ndarray | None = None, vel4: np.ndarray | None = None, visc: float | None = None,
                sigma: float | None = None, stream=None) -> tuple[np.ndarray, np.ndarray]:
        """Sets the initial state / coefficients (when given), runs the recorded forward, returns
        the final state (ID order, float32 (N, 4))."""
        changes = {}
        if visc is not None and float(visc) != self.sim.material["viscosity"]:
            changes["viscosity"] = float(visc)
        if sigma is not None and float(sigma) != self.sim.material["surface_tension"]:
            changes["surface_tension"] = float(sigma)
        if changes:
            self.sim.set_material(**changes)
        if pos4 is not None or vel4 is not None:
            p0, v0 = self.sim.get_fluid(stream)
            self.sim.set_fluid(p0 if pos4 is None else pos4, v0 if vel4 is None else vel4, stream)
        L.check(self.lib.mps_adjoint_forward(self.sim.h, self.nsteps, self.every, stream))
        return self.sim.get_fluid(stream)

    def backward(self, g_pos4: np.ndarray | None, g_vel4: np.ndarray | None, stream=None):
        """Cotangents of the final state -> (d/d pos0, d/d vel0, per-scene [d/d visc, d/d sigma])."""
        n, S = self.sim.n, self.sim.nscenes
        gp = None if g_pos4 is None else np.ascontiguousarray(g_pos4, np.float32).reshape(n, 4)
        gv = None if g_vel4 is None else np.ascontiguousarray(g_vel4, np.float32).reshape(n, 4)
        op = np.zeros((n, 4), np.float32)
        ov = np.zeros((n, 4), np.float32)
        par = np.zeros((S, 2), np.float64)
        L.check(self.lib.mps_adjoint_backward(self.sim.h, None if gp is None else _p(gp), None if gv is None else _p(gv),
                                              _p(op), _p(ov), _p(par), stream))
        return op, ov, par


class _RolloutFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, roll: AdjointRollout, pos0, vel0, visc, sigma):
        p0, v0 = roll.sim.get_fluid()
        p0[:, :3] = pos0.detach().cpu().numpy().astype(np.float32)
        v0[:, :3] = vel0.detach().cpu().numpy().astype(np.float32)
        pT, vT = roll.forward(p0, v0, float(visc), float(sigma))
        ctx.roll = roll
        ctx.dtype = pos0.dtype
        return torch.from_numpy(pT[:, :3].copy()).to(pos0.dtype), torch.from_numpy(vT[:, :3].copy()).to(vel0.dtype)

    @staticmethod
    def backward(ctx, gpos, gvel):
        n = ctx.roll.sim.n
        gp = np.zeros((n, 4), np.float32)
        gv = np.zeros((n, 4), np.float32)
        if gpos is not None:
            gp[:, :3] = gpos.detach().cpu().numpy()
        if gvel is not None:
            gv[:, :3] = gvel.detach().cpu().numpy()
        op, ov, par = ctx.roll.backward(gp, gv)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(ctx.dtype)
        return (None, t(op[:, :3]), t(ov[:, :3]), torch.tensor(par[:, 0].sum(), dtype=ctx.dtype),
                torch.tensor(par[:, 1].sum(), dtype=ctx.dtype))


def rollout(roll: AdjointRollout, pos0: torch.Tensor, vel0: torch.Tensor, visc: torch.Tensor,
            sigma: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Differentiable (pos_T, vel_T) = rollout(pos0, vel0, visc, sigma); tensors on the CPU, (N, 3)."""
    return _RolloutFn.apply(roll, pos0, vel0, visc, sigma)


def com_loss(posT: torch.Tensor, velT: torch.Tensor, mass: torch.Tensor, offsets, targets: torch.Tensor,
             w: float = 1.0e-3) -> torch.Tensor:
    """Per-scene |COM(pos_T) - target|^2 + w mean |vel_T|^2 (COM mass-weighted)."""
    out = []
    for s in range(len(offsets) - 1):
        a, b = int(offsets[s]), int(offsets[s + 1])
        m = mass[a:b, None]
        com = (m * posT[a:b]).sum(0) / m.sum()
        out.append(((com - targets[s]) ** 2).sum() + w * (velT[a:b] ** 2).sum(1).mean())
    return torch.stack(out)
