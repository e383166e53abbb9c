"""Fixed bottom topography, held spectrally on the device.

Mirrors src/planetary_sandbox/physics/topography.py: surface *elevation*
h_s (m) at the model truncation in the dense (l_max+1, l_max+1) complex
layout; ``surface_geopotential_lm(g)`` is phi_s = g h_s.  Presets: ``flat``
(all coefficients exactly zero) and ``mountain`` (one Gaussian mountain
h0 exp(-(d/sigma)^2), d the great-circle distance from its centre, evaluated
on the planet's state points and analysed once with the planet's own
transform; construction fails when the quadrature-weighted relative L2
residual of that projection exceeds 0.2).
"""
from __future__ import annotations

import math

import torch

TOPOGRAPHY_PRESETS = ("flat", "mountain")
MAX_PROJECTION_RESIDUAL = 0.2
MAX_MOUNTAIN_HEIGHT_M = 1.0e5


class TopographyError(ValueError):
    """Invalid topography parameters or coefficients."""


def _require(name, value, *, lo=None, hi=None, positive=False) -> float:
    try:
        x = float(value)
    except (TypeError, ValueError):
        raise TopographyError(f"{name} must be a real number, got {value!r}") from None
    if not math.isfinite(x):
        raise TopographyError(f"{name} must be finite, got {x}")
    if positive and not x > 0:
        raise TopographyError(f"{name} must be > 0, got {x}")
    if lo is not None and x < lo:
        raise TopographyError(f"{name} must be >= {lo}, got {x}")
    if hi is not None and x > hi:
        raise TopographyError(f"{name} must be <= {hi}, got {x}")
    return x


class Topography:
    """Band-limited surface elevation (topography.py:88-292)."""

    def __init__(self, elevation_lm, *, preset: str, parameters: dict | None = None):
        if preset not in TOPOGRAPHY_PRESETS:
            raise TopographyError(f"unknown topography preset {preset!r}; choose from {TOPOGRAPHY_PRESETS}")
        arr = torch.as_tensor(elevation_lm, dtype=torch.complex128)
        if arr.dim() != 2 or arr.shape[0] != arr.shape[1] or arr.shape[0] < 2:
            raise TopographyError("elevation_lm must be a square (l_max+1, l_max+1) array with l_max >= 1, "
                                  f"got shape {tuple(arr.shape)}")
        if not bool(torch.isfinite(torch.view_as_real(arr)).all()):
            raise TopographyError("elevation_lm contains NaN/Inf coefficients")
        self._elevation_lm = arr.clone()
        self._preset = str(preset)
        self._parameters = dict(parameters or {})
        self._l_max = int(arr.shape[0]) - 1
        self._is_flat = not bool((arr != 0).any())
        if preset == "flat" and not self._is_flat:
            raise TopographyError("preset 'flat' requires all elevation coefficients to be zero")

    l_max = property(lambda self: self._l_max)
    preset = property(lambda self: self._preset)
    parameters = property(lambda self: dict(self._parameters))
    is_flat = property(lambda self: self._is_flat)
    elevation_lm = property(lambda self: self._elevation_lm.clone())

    @property
    def mean_elevation_m(self) -> float:
        return float(self._elevation_lm[0, 0].real) / math.sqrt(4.0 * math.pi)

    def describe(self) -> str:
        if self._preset == "mountain":
            p = self._parameters
            return (f"mountain (h={p.get('height_m'):g} m at lat {p.get('lat_deg'):g}°, lon {p.get('lon_deg'):g}°, "
                    f"width {p.get('width_deg'):g}°)")
        return "flat"

    def surface_geopotential_lm(self, gravity: float) -> torch.Tensor:
        """phi_s = g h_s (m^2/s^2), a fresh tensor."""
        return _require("gravity", gravity, positive=True) * self._elevation_lm

    def elevation_on(self, sh) -> torch.Tensor:
        """The band-limited elevation synthesized on ``sh``'s points."""
        return sh.inv_transform(self._elevation_lm.to(sh.weights.device))

    @classmethod
    def flat(cls, l_max: int) -> "Topography":
        if int(l_max) < 1:
            raise TopographyError(f"l_max must be >= 1, got {l_max}")
        n = int(l_max) + 1
        return cls(torch.zeros((n, n), dtype=torch.complex128), preset="flat", parameters={})

    @classmethod
    def mountain(cls, planet, *, height_m: float, lat_deg: float, lon_deg: float, width_deg: float,
                 l_cut: int | None = None) -> "Topography":
        """h0 exp(-(d/sigma)^2) on the state points, analysed with the
        planet's transform (topography.py:207-292); ``l_cut`` zeroes degrees
        and orders above it before the residual gate."""
        height = _require("mountain height_m", height_m, positive=True, hi=MAX_MOUNTAIN_HEIGHT_M)
        lat0 = _require("mountain lat_deg", lat_deg, lo=-90.0, hi=90.0)
        lon0 = _require("mountain lon_deg", lon_deg, lo=-360.0, hi=360.0)
        width = _require("mountain width_deg", width_deg, positive=True, hi=90.0)
        sh = planet.sh
        if l_cut is not None and not 1 <= int(l_cut) <= sh.l_max:
            raise TopographyError(f"l_cut must be in [1, l_max={sh.l_max}], got {l_cut}")
        dev = sh.weights.device
        lat = torch.as_tensor(planet.grid.point_latitudes, dtype=torch.float64, device=dev).reshape(-1)
        lon = torch.as_tensor(planet.grid.point_longitudes, dtype=torch.float64, device=dev).reshape(-1)
        la, lo, sigma = math.radians(lat0), math.radians(lon0), math.radians(width)
        cosd = math.sin(la) * torch.sin(lat) + math.cos(la) * torch.cos(lat) * torch.cos(lon - lo)
        d = torch.arccos(torch.clamp(cosd, -1.0, 1.0))
        analytic = height * torch.exp(-(d / sigma) ** 2)
        coeffs = sh.transform(analytic).to(torch.complex128)
        if not bool(torch.isfinite(torch.view_as_real(coeffs)).all()):
            raise TopographyError("mountain projection produced NaN/Inf coefficients")
        if l_cut is not None:
            coeffs = coeffs.clone()
            coeffs[int(l_cut) + 1:, :] = 0.0
            coeffs[:, int(l_cut) + 1:] = 0.0
        n = sh.l_max + 1
        keep = torch.tril(torch.ones((n, n), dtype=torch.bool, device=coeffs.device))
        coeffs = torch.where(keep, coeffs, torch.zeros((), dtype=coeffs.dtype, device=coeffs.device))
        w = sh.weights.reshape(-1)
        back = sh.inv_transform(coeffs).reshape(-1)
        num = float(torch.sqrt(torch.sum(w * (back - analytic) ** 2)))
        den = float(torch.sqrt(torch.sum(w * analytic ** 2)))
        residual = num / den if den > 0 else math.inf
        if not residual <= MAX_PROJECTION_RESIDUAL:
            raise TopographyError(
                f"mountain (width {width:g}°) is too narrow for l_max={sh.l_max}: projection residual "
                f"{residual:.3g} exceeds {MAX_PROJECTION_RESIDUAL}; widen it or raise l_max")
        params = {"height_m": height, "lat_deg": lat0, "lon_deg": lon0, "width_deg": width,
                  "projection_residual": residual}
        if l_cut is not None:
            params["l_cut"] = int(l_cut)
        return cls(coeffs, preset="mountain", parameters=params)
