"""Initial conditions of ``aeolus run bve|swe`` on the GB300 models.

BVE scenarios (src/planetary_sandbox/run/bve/initial_conditions.py): relative
vorticity on the planet's grid points (reshaped to (nlat, nlon) on
structured grids), which the run analyses with the planet's transform
(cli/bve.py:151-152): pairs of Gaussian vortices exp(-d^2 / (2 sigma^2)),
sigma = 10 deg, amplitude 5e-5 1/s, at mid-latitudes, the poles or the
equator (and their sign-inverted forms); a Rossby-Haurwitz wave 4;
``random_low_l``, random l <= 10 coefficients of amplitude 1e-6 synthesized
on the grid (drawn from torch's generator, so not the reference's draws).

SWE scenarios (run/swe/initial_conditions.py): built spectrally, exactly
monopole-free: ``rest`` (lake at rest over terrain), ``gravity_wave`` (a
Y_4^2 free-surface bump of 1e-3 Phi0) and ``williamson2`` (case 2 wind and
balanced free surface); over topography the thickness perturbation is the
free-surface anomaly minus phi_s'.  Each SWE state is validated before it is
returned.
"""
from __future__ import annotations

import math

import torch

from .shallow_water import ShallowWaterModel, ShallowWaterState


def _latlon(planet):
    dev = planet.sh.weights.device
    lat = torch.as_tensor(planet.grid.point_latitudes, dtype=torch.float64, device=dev).reshape(-1)
    lon = torch.as_tensor(planet.grid.point_longitudes, dtype=torch.float64, device=dev).reshape(-1)
    return lat, lon


def _structured(planet, values):
    shape = getattr(planet.grid, "grid_shape", None)
    if shape is None or len(shape) != 2:
        return values
    if values.numel() != int(shape[0] * shape[1]):
        raise ValueError("values size does not match grid shape")
    return values.reshape(tuple(shape))


def _gaussian(lat, lon, lat0, lon0, sigma):
    cosd = torch.sin(lat) * math.sin(lat0) + torch.cos(lat) * math.cos(lat0) * torch.cos(lon - lon0)
    d = torch.arccos(torch.clamp(cosd, -1.0, 1.0))
    return torch.exp(-(d * d) / (2 * sigma * sigma))


def _pair(planet, sign, c1, c2):
    lat, lon = _latlon(planet)
    s = 10.0 * math.pi / 180.0
    z = sign * 5e-5 * _gaussian(lat, lon, c1[0], c1[1], s)
    z = z + (-sign) * 5e-5 * _gaussian(lat, lon, c2[0], c2[1], s)
    return _structured(planet, z)


_MID = ((33 * math.pi / 180, math.pi / 2), (-33 * math.pi / 180, -math.pi / 2))
_POLE = ((math.pi / 2 - 1e-6, 0.0), (-math.pi / 2 + 1e-6, math.pi))
_EQ = ((0.0, math.pi / 2), (0.0, -math.pi / 2))


def _random_low_l(planet, generator=None):
    L = planet.sh.l_max
    L0 = min(10, L)
    dev = planet.sh.weights.device
    a = torch.zeros((L + 1, L + 1), dtype=torch.complex128, device=dev)
    re = torch.randn((L0 + 1, L0 + 1), dtype=torch.float64, generator=generator)
    im = torch.randn((L0 + 1, L0 + 1), dtype=torch.float64, generator=generator)
    a[:L0 + 1, :L0 + 1] = torch.complex(re, im).to(dev) * 1e-6
    return planet.sh.inv_transform(a)


def _rh4(planet):
    """zeta = 2 nu sin(lat) - 30 K sin(lat) cos^4(lat) sin(4 lon), nu = K = 7.848e-6."""
    lat, lon = _latlon(planet)
    nu = K = 7.848e-6
    sinphi, cosphi = torch.sin(lat), torch.cos(lat)
    zeta = 2.0 * nu * sinphi
    zeta = zeta + -30.0 * K * sinphi * (cosphi ** 4) * torch.sin(4.0 * lon)
    return _structured(planet, zeta)


INITIAL_CONDITIONS = {
    "two_vortices": lambda p: _pair(p, 1.0, *_MID),
    "inverted_vortices": lambda p: _pair(p, -1.0, *_MID),
    "polar_vortices": lambda p: _pair(p, 1.0, *_POLE),
    "inverted_polar_vortices": lambda p: _pair(p, -1.0, *_POLE),
    "equatorial_vortices": lambda p: _pair(p, 1.0, *_EQ),
    "inverted_equatorial_vortices": lambda p: _pair(p, -1.0, *_EQ),
    "random_low_l": _random_low_l,
    "rh4": _rh4,
}


def make_ic(name: str, planet):
    """BVE initial vorticity on the planet's grid (run/bve/initial_conditions.py:110-114)."""
    if name not in INITIAL_CONDITIONS:
        raise ValueError(f"Unknown initial condition: {name}. Available: {list(INITIAL_CONDITIONS.keys())}")
    return INITIAL_CONDITIONS[name](planet)


def _base(model: ShallowWaterModel) -> ShallowWaterState:
    st = ShallowWaterState.zeros(model.l_max, device=model.lap_eigs.device)
    if model.has_topography:
        st.coeffs[2] = -model.phi_s_anom_lm
    return st


def _rest(model):
    st = _base(model)
    model.validate_state(st, context="rest initial condition")
    return st


def _gravity_wave(model):
    l, m = 4, 2
    if model.l_max < l:
        raise ValueError(f"gravity_wave scenario needs l_max >= {l}, got {model.l_max}")
    st = _base(model)
    st.coeffs[2, l, m] += 1e-3 * model.phi0
    model.validate_state(st, context="gravity_wave initial condition")
    return st


def _williamson2(model):
    a, omega = model.R, model.Omega
    u0 = 2.0 * math.pi * a / (12.0 * 86400.0)
    C = a * omega * u0 + 0.5 * u0 * u0
    st = _base(model)
    st.coeffs[0, 1, 0] = (2.0 * u0 / a) * math.sqrt(4.0 * math.pi / 3.0)
    st.coeffs[2, 2, 0] += -(4.0 * C / 3.0) * math.sqrt(math.pi / 5.0)
    model.validate_state(st, context="williamson2 initial condition")
    return st


SWE_INITIAL_CONDITIONS = {"rest": _rest, "gravity_wave": _gravity_wave, "williamson2": _williamson2}


def make_swe_ic(name: str, model: ShallowWaterModel) -> ShallowWaterState:
    """run/swe/initial_conditions.py:111-116."""
    if name not in SWE_INITIAL_CONDITIONS:
        raise ValueError(f"Unknown swe initial condition: {name}. Available: {sorted(SWE_INITIAL_CONDITIONS)}")
    return SWE_INITIAL_CONDITIONS[name](model)


# ---------------------------------------------------------------- PE
THERMAL_WAVE_DEGREE, THERMAL_WAVE_ORDER = 2, 2


def make_pe_ic(name: str, model, *, temperature: float, surface_pressure: float, thermal_amplitude: float = 0.0):
    """Primitive-equation initial states (run/pe/initial_conditions.py), all
    built spectrally on the isothermal rest state: ``isothermal_rest``;
    ``thermal_wave`` (T at (l, m) = (2, 2) set to ``thermal_amplitude`` on every
    level); ``orographic_isothermal_rest`` (ln p_s lowered by
    phi_s / (R_d T0), the balanced rest over the model's terrain)."""
    from .primitive_equations import isothermal_rest_state

    if name not in ("isothermal_rest", "thermal_wave", "orographic_isothermal_rest"):
        raise ValueError(f"Unknown pe initial condition: {name}. "
                         f"Available: {sorted(['isothermal_rest', 'orographic_isothermal_rest', 'thermal_wave'])}")
    dev = model.phi_surface_lm.device
    st = isothermal_rest_state(model.l_max, model.nlev, temperature=temperature,
                               surface_pressure=surface_pressure, device=dev)
    if name == "thermal_wave":
        if model.l_max < THERMAL_WAVE_DEGREE:
            raise ValueError(f"thermal_wave needs l_max >= {THERMAL_WAVE_DEGREE}, got {model.l_max}")
        st.coeffs[2 * model.nlev:3 * model.nlev, THERMAL_WAVE_DEGREE, THERMAL_WAVE_ORDER] = float(thermal_amplitude)
    elif name == "orographic_isothermal_rest":
        st.coeffs[3 * model.nlev] -= model.phi_surface_lm / (model.r_dry * float(temperature))
    return st
