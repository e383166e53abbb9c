"""Seeded synthetic inputs for the benchmark and parity workloads.

Every workload here is synthetic (there is no public dataset for this path);
the generators follow the published input recipes of the workloads:

* small BVE: Gauss 32x64, l_max=21, vorticity coefficients with real and
  imaginary parts ~ N(0,1) (l+1)^-1.5 1e-5 s^-1, Im = 0 at m = 0, l = 0 zero;
* shallow water: Williamson-2 base state (u0 = 2 pi a / 12 days,
  g h0 = 2.94e4 m^2/s^2) plus a seeded perturbation per field
  ~ N(0,1) (l+1)^-2 scaled to 1 % of the base-state RMS (divergence, whose
  base RMS is zero, is scaled to 1 % of the vorticity base RMS);
* geodesic batch: fields ~ N(0,1) (l+1)^-1.5.

All arrays use the reference's dense (l_max+1, l_max+1) complex layout
(axis 0 = degree l, axis 1 = order m, m > l slots zero).
"""
from __future__ import annotations

import math

import numpy as np

EARTH_RADIUS = 6.371e6          # m
EARTH_OMEGA = 7.292e-5          # 1/s
GRAVITY = 9.80616               # m/s^2, Williamson et al. (1992)
GH0 = 2.94e4                    # m^2/s^2


def triangle_mask(lmax: int) -> np.ndarray:
    l = np.arange(lmax + 1)
    return l[None, :] <= l[:, None]


def random_spectrum(rng: np.random.Generator, lmax: int, slope: float,
                    amp: float = 1.0, zero_monopole: bool = True) -> np.ndarray:
    """Coefficients of a real field: a_lm ~ N(0,1)(l+1)^slope amp, Im a_l0 = 0."""
    n = lmax + 1
    re = rng.standard_normal((n, n))
    im = rng.standard_normal((n, n))
    scale = amp * (np.arange(n, dtype=np.float64) + 1.0) ** slope
    a = (re + 1j * im) * scale[:, None]
    a[:, 0] = a[:, 0].real
    if zero_monopole:
        a[0, :] = 0.0
    a[~triangle_mask(lmax)] = 0.0
    return a


def spectral_rms(a: np.ndarray) -> float:
    """Area RMS of the synthesized field, sqrt(sum of mode power / 4 pi)."""
    lmax = a.shape[0] - 1
    p = np.where(np.arange(lmax + 1)[None, :] == 0, a.real ** 2, 2.0 * np.abs(a) ** 2)
    p = np.where(triangle_mask(lmax), p, 0.0)
    return float(np.sqrt(p.sum() / (4.0 * math.pi)))


def bve_vorticity(lmax: int, seed: int = 0) -> np.ndarray:
    """Small-BVE vorticity spectrum (1e-5 s^-1 amplitude, slope -1.5)."""
    return random_spectrum(np.random.default_rng(seed), lmax, -1.5, 1e-5)


def williamson2(lmax: int, radius: float = EARTH_RADIUS, omega: float = EARTH_OMEGA,
                gravity: float = GRAVITY, gh0: float = GH0):
    """Williamson case-2 state (3, L+1, L+1) and the mean depth H.

    Follows src/planetary_sandbox/run/swe/initial_conditions.py:74-101:
    zeta[1,0] = (2 u0/a) sqrt(4 pi/3), phi[2,0] = -(4C/3) sqrt(pi/5),
    C = a Omega u0 + u0^2/2; H = (g h0 - C/3)/g (tests/test_williamson2.py:65).
    """
    u0 = 2.0 * math.pi * radius / (12.0 * 86400.0)
    C = radius * omega * u0 + 0.5 * u0 * u0
    s = np.zeros((3, lmax + 1, lmax + 1), dtype=np.complex128)
    s[0, 1, 0] = (2.0 * u0 / radius) * math.sqrt(4.0 * math.pi / 3.0)
    s[2, 2, 0] = -(4.0 * C / 3.0) * math.sqrt(math.pi / 5.0)
    return s, (gh0 - C / 3.0) / gravity


def perturbed_williamson2(lmax: int, seed: int, radius: float = EARTH_RADIUS,
                          omega: float = EARTH_OMEGA, gravity: float = GRAVITY,
                          rel: float = 0.01):
    """Williamson-2 plus a seeded (l+1)^-2 perturbation at `rel` of base RMS."""
    base, depth = williamson2(lmax, radius, omega, gravity)
    rng = np.random.default_rng(seed)
    out = base.copy()
    for f in range(3):
        p = random_spectrum(rng, lmax, -2.0, 1.0)
        ref = spectral_rms(base[f]) if f != 1 else spectral_rms(base[0])
        out[f] += (rel * ref / spectral_rms(p)) * p
    return out, depth


def member_states(lmax: int, members: int, seed: int, **kw):
    """`members` independent perturbed Williamson-2 states, (B, 3, L+1, L+1)."""
    states = []
    depth = None
    for b in range(members):
        s, depth = perturbed_williamson2(lmax, seed + 1000 * b, **kw)
        states.append(s)
    return np.stack(states), depth
