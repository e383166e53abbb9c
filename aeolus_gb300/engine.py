"""Generic RK4 for stacked coefficient arrays, src/planetary_sandbox/run/engine.py:406-431.

For the BVE and SWE models prefer ``model.rk4`` (all stages fused on the
device); this form accepts any tendency callable and an optional stage
validator, exactly like the reference.
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
