"""Generic RK4 for stacked coefficient arrays, src/planetary_sandbox/run/engine.py:406-431.

For the BVE and SWE models prefer ``model.rk4`` (all stages fused on the
device); this form accepts any tendency callable and an optional stage
validator, exactly like the reference.  ``rk4_step_device`` is the same step
with the stage combinations fused on the device.
"""
from __future__ import annotations


def rk4_step_array(tendency, y, t: float, dt: float, *, stage_validator=None):
    def _stage(ys):
        if stage_validator is not None:
            stage_validator(ys)
        return ys

    k1 = tendency(y)
    k2 = tendency(_stage(y + 0.5 * dt * k1))
    k3 = tendency(_stage(y + 0.5 * dt * k2))
    k4 = tendency(_stage(y + dt * k3))
    return y + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)


def rk4_step_device(tendency, y, t: float, dt: float, *, stage_validator=None):
    """rk4_step_array with the stage combinations fused on the device (one
    aeolus_rk4_stage launch per stage instead of the elementwise torch
    operations), the same order of operations and rounding: bitwise the
    same step.  `y` is a complex128 CUDA tensor; the tendency returns one of
    the same shape."""
    import torch

    from .ops import rk4_stage

    y0 = y.contiguous()
    ys = torch.empty_like(y0)
    acc = torch.empty_like(y0)
    for stage in (1, 2, 3, 4):
        k = tendency(y0 if stage == 1 else ys).contiguous()
        rk4_stage(stage, dt, y0, k, ys, acc)
        if stage < 4 and stage_validator is not None:
            stage_validator(ys)
    return ys
