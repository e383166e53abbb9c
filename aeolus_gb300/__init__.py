"""aeolus_gb300 -- GB300 (sm_103a) spectral hot path of the Aeolus laboratory.

Spherical-harmonic synthesis/analysis (Gauss-Legendre: per-order Legendre
contraction + longitude real FFT; point sets: dense basis product) and the
barotropic-vorticity / shallow-water tendencies and RK4 steps built on them,
behind the reference's backend and operator API.  Compute runs in the
in-tree C-ABI library ``libaeolus_gb300.so`` (see include/aeolus_gb300.h);
there is no CPU fallback.
"""
from __future__ import annotations

from types import SimpleNamespace

__version__ = "0.1.0"


def make_planet(grid_type: str = "latlon", *, nlat: int = 32, nlon: int = 64, l_max: int = 21,
                resolution: int = 4, radius: float = 6.371e6, omega: float = 7.292e-5,
                product_quadrature: str = "fine", device=None):
    """The (sh, so, grid, params) bundle the models consume, built directly
    with explicit constants (the reference's Planet.generate also makes
    decorative terrain and derives its own radius and rotation rate)."""
    from .latlon_grid import GaussLatLonGridGeometry, GaussLatLonSphericalHarmonics
    from .geodesic_grid import GeodesicGridGeometry, GeodesicSphericalHarmonics
    from .spherical_backend import make_backend
    from .spectral_operators import SpectralOperators

    if grid_type == "latlon":
        grid = GaussLatLonGridGeometry(nlat, nlon, radius, device)
        sh = GaussLatLonSphericalHarmonics(grid, l_max)
    elif grid_type == "geodesic":
        grid = GeodesicGridGeometry(resolution, radius, device)
        sh = GeodesicSphericalHarmonics(grid, l_max, weights="voronoi")
    else:
        raise ValueError(f"unknown grid_type {grid_type!r} (expected 'latlon' or 'geodesic')")
    backend = make_backend(grid, sh)
    so = SpectralOperators(sh, radius, grid, product_quadrature=product_quadrature, backend=backend)
    return SimpleNamespace(sh=sh, so=so, grid=grid, params=SimpleNamespace(radius=radius, angular_velocity=omega))
