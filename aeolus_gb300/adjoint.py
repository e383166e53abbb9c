"""Differentiation through the spectral models: hand-written adjoints behind
``torch.autograd.Function``.

The reference has no gradients; this module adds them on top of the GB300
kernels.  Every backward is a call into ``libaeolus_gb300.so``:

* ``synthesize`` / ``analyze`` (``aeolus_gb300.ops``) carry registered
  autograd formulas whose backward is the transposed transform
  (``aeolus_synthesize_adjoint`` = unit-weight analysis with the m > 0
  factor 2, ``aeolus_analyze_adjoint`` = weighted synthesis of the halved
  m > 0 slots).
* :func:`swe_rk4_checkpointed` / :func:`bve_rk4_checkpointed` advance
  ``nsteps`` RK4 steps and keep the step input every ``every`` steps; their
  backward re-runs each segment forward from its checkpoint (holding the
  ``every`` step inputs of one segment) and applies the per-step adjoint
  (``aeolus_swe_rk4_adjoint``), which recomputes the stage inputs and runs
  the four tendency VJPs on the device.

Peak device memory is therefore (checkpoints + one segment) states plus one
RK4-adjoint workspace, independent of ``nsteps``.
"""
from __future__ import annotations

import torch

from .ops import bve_rk4_adjoint, swe_rk4_adjoint


class _SweRk4Checkpointed(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y0, model, dt, nsteps, every):
        every = max(1, int(every))
        ckpts = []
        y = y0.detach()
        for i in range(nsteps):
            if i % every == 0:
                ckpts.append(y.clone())
            y = model.rk4(y, dt, 1, check=False)
        ctx.model, ctx.dt, ctx.nsteps, ctx.every, ctx.ckpts = model, float(dt), int(nsteps), every, ckpts
        return y

    @staticmethod
    def backward(ctx, ybar):
        m = ctx.model
        yb = ybar.contiguous()
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            start = seg * ctx.every
            n = min(ctx.every, ctx.nsteps - start)
            states = [ctx.ckpts[seg]]
            for _ in range(n - 1):
                states.append(m.rk4(states[-1], ctx.dt, 1, check=False))
            for i in range(n - 1, -1, -1):
                yb = swe_rk4_adjoint(m._plan.id, m.R, m.Omega, m.gravity, m.mean_depth, m.nu4, states[i], yb, ctx.dt,
                                     m.forcing)
        return yb, None, None, None, None


class _BveRk4Checkpointed(torch.autograd.Function):
    @staticmethod
    def forward(ctx, z0, model, dt, nsteps, every):
        every = max(1, int(every))
        ckpts = []
        z = z0.detach()
        for i in range(nsteps):
            if i % every == 0:
                ckpts.append(z.clone())
            z = model.rk4(z, dt, 1)
        ctx.model, ctx.dt, ctx.nsteps, ctx.every, ctx.ckpts = model, float(dt), int(nsteps), every, ckpts
        return z

    @staticmethod
    def backward(ctx, zbar):
        m = ctx.model
        zb = zbar.contiguous()
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            start = seg * ctx.every
            n = min(ctx.every, ctx.nsteps - start)
            states = [ctx.ckpts[seg]]
            for _ in range(n - 1):
                states.append(m.rk4(states[-1], ctx.dt, 1))
            for i in range(n - 1, -1, -1):
                zb = bve_rk4_adjoint(m._plan.id, m.R, m.Omega, m.nu, states[i], zb, ctx.dt)
        return zb, None, None, None, None


def swe_rk4_checkpointed(model, y0: torch.Tensor, dt: float, nsteps: int, every: int = 8) -> torch.Tensor:
    """``nsteps`` SWE RK4 steps of ``[..., 3, L+1, L+1]`` states, differentiable
    in ``y0`` through the hand-written adjoint with checkpoints every
    ``every`` steps (run/engine.py:406-431 differentiated)."""
    return _SweRk4Checkpointed.apply(y0, model, float(dt), int(nsteps), int(every))


def bve_rk4_checkpointed(model, z0: torch.Tensor, dt: float, nsteps: int, every: int = 8) -> torch.Tensor:
    """``nsteps`` BVE RK4 steps, differentiable in ``z0`` (run/bve/runner.py:211-216)."""
    return _BveRk4Checkpointed.apply(z0, model, float(dt), int(nsteps), int(every))


def weighted_phi_misfit(model, y: torch.Tensor, target_grid: torch.Tensor) -> torch.Tensor:
    """Area-weighted squared error of the final geopotential on the state
    grid: sum_points w (phi(y) - target)^2 per member (w = the quadrature
    weights, summing to 4 pi).  Differentiable through ``synthesize``."""
    from .ops import synthesize
    plan = model._state_plan
    g = synthesize(plan.id, y[..., 2, :, :])
    w = model.sh.weights.reshape(-1).to(g)
    return ((g - target_grid) ** 2 * w).sum(dim=-1)
