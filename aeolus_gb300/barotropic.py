"""Barotropic vorticity equation on the GB300 path.

Mirrors src/planetary_sandbox/physics/barotropic.py:14-197 and the RK4 of
src/planetary_sandbox/run/bve/runner.py:211-216.  ``tendency`` is one fused
chain on the product space (derivative coefficients -> synthesis -> Jacobian
-> analysis -> 2/3 cut + viscosity + l=0 pin); ``rk4_step`` advances whole
steps with no host round trips.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from . import _lib
from .ops import bve_rk4, bve_tendency, spectral_op


@dataclass
class BarotropicState:
    coeffs: torch.Tensor
    tendency: torch.Tensor | None = None


class BarotropicVorticity:
    """dζ/dt = -J(ψ, ζ + f) + ν ∇²ζ (+ F), l = 0 row pinned."""

    def __init__(self, planet, scenario: str = "two_vortices", viscosity: float = 0.0):
        self.planet = planet
        self.nu = float(viscosity)
        self.sh = planet.sh
        self.so = planet.so
        self.grid = planet.grid
        self.R = float(planet.params.radius)
        self.Omega = float(planet.params.angular_velocity)
        lat = torch.as_tensor(self.grid.point_latitudes)
        f = 2 * self.Omega * torch.sin(lat)
        shape = getattr(self.grid, "grid_shape", None)
        if shape is not None and len(shape) == 2 and f.numel() == int(shape[0] * shape[1]):
            f = f.reshape(shape)
        self.f = f
        L = self.sh.l_max
        dev = lat.device
        self.f_lm = torch.zeros((L + 1, L + 1), dtype=torch.complex128, device=dev)
        self.f_lm[1, 0] = 2.0 * self.Omega * math.sqrt(4.0 * math.pi / 3.0)
        l = torch.arange(L + 1, dtype=torch.float64, device=dev)
        self.laplacian_eig = -l * (l + 1) / self.R ** 2
        self.laplacian_eig[0] = 1.0 / self.R ** 2
        self._plan = self.so._product_space.sh.plan

    def vorticity_to_streamfunction(self, vrt_state: BarotropicState) -> torch.Tensor:
        """ψ = ∇⁻²ζ with the l = 0 row zero, barotropic.py:68-93."""
        assert isinstance(vrt_state, BarotropicState)
        return spectral_op(_lib.SOP_INV_LAPLACIAN_ZERO, self.R, vrt_state.coeffs)

    def streamfunction_to_vorticity(self, psi_coeffs) -> BarotropicState:
        """ζ = ∇²ψ (l = 0 row zero), barotropic.py:95-117."""
        return BarotropicState(spectral_op(_lib.SOP_LAPLACIAN, self.R, psi_coeffs))

    def tendency(self, vrt_state: BarotropicState, forcing_coeffs=None) -> torch.Tensor:
        return bve_tendency(self._plan.id, self.R, self.Omega, self.nu, vrt_state.coeffs, forcing_coeffs)

    def rk4(self, zeta: torch.Tensor, dt: float, nsteps: int = 1) -> torch.Tensor:
        """nsteps fused RK4 steps (all stages on the device)."""
        return bve_rk4(self._plan.id, self.R, self.Omega, self.nu, zeta, float(dt), int(nsteps))


def rk4_step(model: BarotropicVorticity, y: BarotropicState, t: float, dt: float,
             forcing_coeffs=None) -> BarotropicState:
    """Classical RK4, run/bve/runner.py:211-216."""
    if forcing_coeffs is None:
        return BarotropicState(model.rk4(y.coeffs, dt, 1))
    k1 = model.tendency(y, forcing_coeffs)
    k2 = model.tendency(BarotropicState(y.coeffs + 0.5 * dt * k1), forcing_coeffs)
    k3 = model.tendency(BarotropicState(y.coeffs + 0.5 * dt * k2), forcing_coeffs)
    k4 = model.tendency(BarotropicState(y.coeffs + dt * k3), forcing_coeffs)
    return BarotropicState(y.coeffs + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4))
