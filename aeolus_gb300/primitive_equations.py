"""Dry hydrostatic primitive equations on the GB300 path.

Mirrors src/planetary_sandbox/physics/sigma_coordinate.py:38-149 (the
Lorenz sigma grid) and physics/primitive_equations.py:40-753 (state layout,
isothermal rest state, model constructor checks and the explicit tendency).
The tendency runs on the device, batched over levels and members:

  aeolus_pe_derive    spectral derivative fields of every level
  aeolus_synthesize   10 K + 2 fields per member on the product plan
  aeolus_pe_columns   the vertical column physics at every product point
  aeolus_analyze      4 K + 1 integrands per member
  aeolus_vector_curl_div  weak-form curl/div of Z on the extended plan
  aeolus_pe_spectral  2/3 cuts, Simmons-Burridge geopotential, l = 0 pins
"""
from __future__ import annotations

import math
from ctypes import byref, c_void_p
from dataclasses import dataclass
from functools import cached_property

import numpy as np
import torch

from . import _lib
from ._lib import check
from .ops import analyze, spectral_op, synthesize, vector_curl_div, winds

R_DRY = 287.04          # J kg^-1 K^-1, primitive_equations.py:49
CP_DRY = 1004.64        # J kg^-1 K^-1
KAPPA_DRY = R_DRY / CP_DRY
MAX_LEVELS = 64
PROGNOSTICS = ("zeta", "delta", "temperature", "ln_ps")


class SigmaGridError(ValueError):
    """The vertical-grid metadata violated a hard structural constraint."""


def product_truncation_cut(l_max: int) -> int:
    return (2 * int(l_max)) // 3


@dataclass(frozen=True)
class SigmaGrid:
    """Interfaces sigma_{k+1/2} top to bottom, exactly 0.0 .. exactly 1.0
    (sigma_coordinate.py:43-149)."""

    interfaces: tuple

    def __post_init__(self):
        try:
            s = tuple(float(x) for x in self.interfaces)
        except (TypeError, ValueError):
            raise SigmaGridError(f"sigma interfaces must be real numbers, got {self.interfaces!r}") from None
        if len(s) < 2:
            raise SigmaGridError("need at least two sigma interfaces (one layer)")
        if not all(math.isfinite(x) for x in s):
            raise SigmaGridError(f"sigma interfaces must be finite, got {s}")
        if s[0] != 0.0 or s[-1] != 1.0:
            raise SigmaGridError(f"sigma interfaces must start at exactly 0.0 and end at exactly 1.0, got {s}")
        if any(b <= a for a, b in zip(s, s[1:])):
            raise SigmaGridError(f"sigma interfaces must be strictly increasing, got {s}")
        if len(s) - 1 > MAX_LEVELS:
            raise SigmaGridError(f"at most {MAX_LEVELS} levels on the GB300 path, got {len(s) - 1}")
        object.__setattr__(self, "interfaces", s)

    @classmethod
    def uniform(cls, nlev: int) -> "SigmaGrid":
        if not isinstance(nlev, int) or isinstance(nlev, bool) or nlev < 1:
            raise SigmaGridError(f"nlev must be a positive int, got {nlev!r}")
        return cls(tuple(k / nlev for k in range(nlev + 1)))

    @property
    def nlev(self) -> int:
        return len(self.interfaces) - 1

    @cached_property
    def full_levels(self):
        s = self.interfaces
        return tuple(0.5 * (s[k] + s[k + 1]) for k in range(self.nlev))

    @cached_property
    def thickness(self):
        s = self.interfaces
        return tuple(s[k + 1] - s[k] for k in range(self.nlev))

    @cached_property
    def interface_log_ratios(self):
        s = self.interfaces
        return (math.inf,) + tuple(math.log(s[k + 1] / s[k]) for k in range(1, self.nlev))

    @cached_property
    def alpha(self):
        s = self.interfaces
        return (math.log(2.0),) + tuple(1.0 - (s[k] / self.thickness[k]) * self.interface_log_ratios[k]
                                        for k in range(1, self.nlev))

    def interfaces_array(self) -> np.ndarray:
        return np.asarray(self.interfaces, dtype=np.float64)


class PrimitiveEquationsStateError(ValueError):
    """A primitive-equation state violated a hard constraint."""


@dataclass
class PrimitiveEquationsState:
    """One (3 nlev + 1, l_max + 1, l_max + 1) complex stack (:76-136)."""

    coeffs: torch.Tensor

    def __post_init__(self):
        c = self.coeffs
        if c.dim() != 3 or (c.shape[0] - 1) % 3 != 0 or c.shape[0] < 4 or c.shape[1] != c.shape[2]:
            raise PrimitiveEquationsStateError(
                f"primitive-equation coefficients must have shape (3*nlev+1, l_max+1, l_max+1) with nlev >= 1, "
                f"got {tuple(c.shape)}")

    nlev = property(lambda self: (self.coeffs.shape[0] - 1) // 3)
    zeta = property(lambda self: self.coeffs[0:self.nlev])
    delta = property(lambda self: self.coeffs[self.nlev:2 * self.nlev])
    temperature = property(lambda self: self.coeffs[2 * self.nlev:3 * self.nlev])
    ln_ps = property(lambda self: self.coeffs[3 * self.nlev])

    @classmethod
    def from_fields(cls, zeta_lm, delta_lm, temperature_lm, ln_ps_lm) -> "PrimitiveEquationsState":
        parts = [torch.as_tensor(a, dtype=torch.complex128) for a in (zeta_lm, delta_lm, temperature_lm)]
        return cls(torch.cat(parts + [torch.as_tensor(ln_ps_lm, dtype=torch.complex128)[None]], dim=0))

    @classmethod
    def zeros(cls, l_max: int, nlev: int, device=None) -> "PrimitiveEquationsState":
        n = l_max + 1
        return cls(torch.zeros((3 * nlev + 1, n, n), dtype=torch.complex128, device=device or "cuda"))


def isothermal_rest_state(l_max: int, nlev: int, *, temperature: float, surface_pressure: float,
                          device=None) -> PrimitiveEquationsState:
    """zeta = delta = 0, T_k = temperature, p_s = surface_pressure (:139-161)."""
    if not (math.isfinite(temperature) and temperature > 0):
        raise ValueError(f"temperature must be finite and > 0, got {temperature}")
    if not (math.isfinite(surface_pressure) and surface_pressure > 0):
        raise ValueError(f"surface_pressure must be finite and > 0, got {surface_pressure}")
    st = PrimitiveEquationsState.zeros(l_max, nlev, device)
    mono = math.sqrt(4.0 * math.pi)
    st.coeffs[2 * nlev:3 * nlev, 0, 0] = temperature * mono
    st.coeffs[3 * nlev, 0, 0] = math.log(surface_pressure) * mono
    return st


def _p(t: torch.Tensor | None) -> c_void_p:
    return c_void_p(0 if t is None else t.data_ptr())


class PrimitiveEquationsModel:
    """Explicit dry hydrostatic PE tendency, primitive_equations.py:164-753
    (full T, no semi-implicit split, no hyperdiffusion)."""

    def __init__(self, planet, sigma: SigmaGrid, *, r_dry: float = R_DRY, cp_dry: float = CP_DRY,
                 surface_geopotential_lm=None):
        if not (math.isfinite(r_dry) and r_dry > 0):
            raise ValueError(f"r_dry must be finite and > 0, got {r_dry}")
        if not (math.isfinite(cp_dry) and cp_dry > r_dry):
            raise ValueError(f"cp_dry must be finite and > r_dry, got {cp_dry}")
        self.planet, self.sh, self.so, self.grid = planet, planet.sh, planet.so, planet.grid
        self.R = float(planet.params.radius)
        self.Omega = float(planet.params.angular_velocity)
        self.sigma = sigma
        self.nlev = sigma.nlev
        self.r_dry, self.cp_dry = float(r_dry), float(cp_dry)
        self.kappa = self.r_dry / self.cp_dry
        self.gamma = self.cp_dry / (self.cp_dry - self.r_dry)
        self.l_max = self.sh.l_max
        n = self.l_max + 1
        dev = self.sh.weights.device
        self._phi_cut = product_truncation_cut(self.l_max)
        if surface_geopotential_lm is None:
            phi_s = torch.zeros((n, n), dtype=torch.complex128, device=dev)
        else:
            phi_s = torch.as_tensor(surface_geopotential_lm, dtype=torch.complex128, device=dev)
            if tuple(phi_s.shape) != (n, n):
                raise ValueError(f"surface_geopotential_lm must have shape {(n, n)}, got {tuple(phi_s.shape)}")
            if not bool(torch.isfinite(phi_s).all()):
                raise ValueError("surface_geopotential_lm contains NaN/Inf")
            cut = self._phi_cut
            if bool((phi_s[cut + 1:, :] != 0).any()) or bool((phi_s[:, cut + 1:] != 0).any()):
                raise ValueError(
                    f"surface_geopotential_lm has spectral content above the dealiased product truncation "
                    f"l = {cut} (2*l_max/3 for l_max = {self.l_max}); band-limit the terrain at the cut")
        self.phi_surface_lm = phi_s.contiguous()
        self._ps = self.so.backend.product_space(self.so.product_quadrature)
        self._plan = self._ps.sh.plan
        self._params = _lib.PeParams(self.R, self.Omega, self.r_dry, self.cp_dry)
        self._sigma_host = np.ascontiguousarray(sigma.interfaces_array())

    def _ext_plan(self):
        return self.so._extended_plan()

    def tendency(self, coeffs: torch.Tensor) -> torch.Tensor:
        """d/dt of the (..., 3K+1, L+1, L+1) stack (:727-753)."""
        K, L = self.nlev, self.l_max
        n = L + 1
        c = torch.as_tensor(coeffs)
        if not c.is_cuda:
            raise ValueError("primitive-equation state must be a CUDA tensor (no CPU fallback)")
        if tuple(c.shape[-3:]) != (3 * K + 1, n, n):
            raise PrimitiveEquationsStateError(
                f"expected [..., {3 * K + 1}, {n}, {n}] coefficients for nlev={K}, l_max={L}, got {tuple(c.shape)}")
        lead = tuple(c.shape[:-3])
        x = c.to(torch.complex128).contiguous().reshape(-1, 3 * K + 1, n, n)
        B = x.shape[0]
        out = torch.empty_like(x)
        if B == 0:
            return out.reshape(lead + (3 * K + 1, n, n))
        lib = _lib.load()
        dev = x.device
        stream = c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        plan = self._plan
        fields = torch.empty((B, 10 * K + 2, n, n), dtype=torch.complex128, device=dev)
        check(lib.aeolus_pe_derive(plan.handle, byref(self._params), K, _p(x), _p(fields), B, stream))
        grid = synthesize(plan.id, fields)                                  # [B, 10K+2, np]
        npts = grid.shape[-1]
        prod = torch.empty((B, 4 * K + 1, npts), dtype=torch.float64, device=dev)
        fen = torch.empty((B * K, 2, npts), dtype=torch.float64, device=dev)
        sig = self._sigma_host
        check(lib.aeolus_pe_columns(plan.handle, byref(self._params), K, sig.ctypes.data_as(c_void_p), _p(grid),
                                    _p(prod), _p(fen), B, stream))
        an = analyze(plan.id, prod)                                         # [B, 4K+1, n, n]
        ext = self._ext_plan()
        cd = vector_curl_div(ext.id, self.R, fen[:, 0], fen[:, 1], False)   # [2, B*K, n, n]
        curl_z, div_z = cd[0].contiguous(), cd[1].contiguous()
        check(lib.aeolus_pe_spectral(L, byref(self._params), K, sig.ctypes.data_as(c_void_p), _p(x), _p(an),
                                     _p(curl_z), _p(div_z), _p(self.phi_surface_lm), _p(out), B, stream))
        return out.reshape(lead + (3 * K + 1, n, n))

    def tendency_state(self, state: PrimitiveEquationsState) -> PrimitiveEquationsState:
        return PrimitiveEquationsState(self.tendency(state.coeffs))

    def rk4(self, coeffs: torch.Tensor, dt: float, nsteps: int = 1, *, stage_validator=None) -> torch.Tensor:
        """`nsteps` classical RK4 steps of the (..., 3K+1, L+1, L+1) stack, each
        the reference's rk4_step_array (run/engine.py:406-431, as the PE runner
        uses it, run/pe/runner.py:104) with its stage combinations fused on the
        device (aeolus_rk4_stage): bitwise the generic engine's step."""
        from .engine import rk4_step_device

        y = torch.as_tensor(coeffs).to(torch.complex128).contiguous()
        for _ in range(int(nsteps)):
            y = rk4_step_device(self.tendency, y, 0.0, dt, stage_validator=stage_validator)
        return y

    # -- state-grid reconstructions, characteristic speed, validation ------
    def wind_on_state_grid(self, state: PrimitiveEquationsState):
        """Per-level (u, v) on the state sampling, (nlev, n_points) each (:289-307)."""
        psi = spectral_op(_lib.SOP_INV_LAPLACIAN_ZERO, self.R, state.zeta)
        chi = spectral_op(_lib.SOP_INV_LAPLACIAN_ZERO, self.R, state.delta)
        uv = winds(self.sh.plan.id, self.R, psi, chi)           # [2, nlev, n_points]
        return uv[0], uv[1]

    def temperature_on_state_grid(self, state: PrimitiveEquationsState) -> torch.Tensor:
        return synthesize(self.sh.plan.id, state.temperature)

    def surface_pressure_on_state_grid(self, state: PrimitiveEquationsState) -> torch.Tensor:
        return torch.exp(synthesize(self.sh.plan.id, state.ln_ps))

    def temperature_extrema(self, state: PrimitiveEquationsState):
        """(min, max) of T over every level on the state and product samplings (:764-781)."""
        plans = [self.sh.plan] + ([self._plan] if self._plan is not self.sh.plan else [])
        ext = torch.stack([torch.stack(torch.aminmax(synthesize(p.id, state.temperature))) for p in plans])
        lo, hi = ext[:, 0].min(), ext[:, 1].max()
        return float(lo), float(hi)

    def max_characteristic_speed(self, state: PrimitiveEquationsState) -> float:
        """max_k max|V_k| + sqrt(gamma R_d T_max) (:783-797)."""
        u, v = self.wind_on_state_grid(state)
        wind_max = float(torch.sqrt(u * u + v * v).max())
        _, t_max = self.temperature_extrema(state)
        return wind_max + math.sqrt(self.gamma * self.r_dry * max(t_max, 0.0))

    _MONOPOLE_RTOL = 1e-10

    def validate_state(self, state: PrimitiveEquationsState, *, context: str = "") -> None:
        """Raise PrimitiveEquationsStateError on a hard violation (:808-854):
        shape, NaN/Inf, per-level zeta/delta monopoles, T > 0 over the state
        and product samplings, finite exp(ln p_s) on the state grid."""
        where = f" {context}" if context else ""
        n = self.l_max + 1
        expected = (3 * self.nlev + 1, n, n)
        if tuple(state.coeffs.shape) != expected:
            raise PrimitiveEquationsStateError(
                f"state shape {tuple(state.coeffs.shape)} does not match the model's expected {expected}{where}")
        if not bool(torch.isfinite(torch.view_as_real(state.coeffs)).all()):
            raise PrimitiveEquationsStateError(f"primitive-equation state contains NaN/Inf coefficients{where}")
        for name, stack in (("zeta", state.zeta), ("delta", state.delta)):
            mono = stack[:, 0, 0].abs()
            scale = torch.linalg.vector_norm(stack.reshape(self.nlev, -1), dim=1)
            bad = (mono > self._MONOPOLE_RTOL * torch.clamp(scale, min=1e-30)).nonzero()
            if bad.numel():
                k = int(bad[0, 0])
                raise PrimitiveEquationsStateError(
                    f"{name} monopole is nonzero at level {k + 1}{where}: |a00| = {float(mono[k]):g} "
                    f"(field norm {float(scale[k]):g}); the global mean of {name} must stay exactly zero on every "
                    "level")
        t_min, _ = self.temperature_extrema(state)
        if not (t_min > 0.0):
            raise PrimitiveEquationsStateError(
                f"temperature is not strictly positive{where}: min(T) = {t_min:g} K over the state/product "
                "samplings")
        if not bool(torch.isfinite(self.surface_pressure_on_state_grid(state)).all()):
            raise PrimitiveEquationsStateError(
                f"surface pressure exp(ln p_s) overflowed to a non-finite value on the state grid{where}")
