"""Icosahedral geodesic point set and the point-set transforms.

Mirrors src/planetary_sandbox/numerics/geodesic_grid.py (geometry, point
order, Voronoi areas), numerics/fast_geodesic_sh.py
(``PointSetSphericalHarmonics``) and numerics/optimized_geodesic_sh.py
(``GeodesicSphericalHarmonics`` with "voronoi" / "uniform" / explicit
weights).  The geometry is built on the device (``csrc/geodesic.cu``); the transform
is a dense real basis built and contracted on the device
(``csrc/points.cu``).
"""
from __future__ import annotations

import warnings

import numpy as np
import torch

from .ops import Plan, analyze, geodesic_build, synthesize

MIN_POINTS_PER_BASIS = 6  # optimized_geodesic_sh.py:23


class GeodesicGridGeometry:
    """Icosahedral geodesic grid, geodesic_grid.py:11-266, built on the
    device (``aeolus_geodesic_build``): the subdivision keeps the reference's
    point and face order, the cell areas are its barycentric "Voronoi"
    areas.  ``points`` and ``faces`` are also kept as host arrays, as the
    reference exposes them."""

    def __init__(self, resolution: int = 0, radius: float = 1.0, device=None):
        self.resolution = int(resolution)
        self.radius = float(radius)
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        g = geodesic_build(self.resolution, self.radius, self.device)
        self.points = g["points"].cpu().numpy()
        self.faces = g["faces"].cpu().numpy()
        self.n_points = len(self.points)
        self.n_faces = len(self.faces)
        self.min_edge_length = g["min_edge"]
        self.latitudes = g["lat"]
        self.longitudes = g["lon"]
        self._lat_np = self.latitudes.cpu().numpy()
        self._lon_np = self.longitudes.cpu().numpy()
        self.sinlat = torch.sin(self.latitudes)
        self.coslat = torch.cos(self.latitudes)
        self._cell_areas = g["areas"]

    point_latitudes = property(lambda self: self.latitudes)
    point_longitudes = property(lambda self: self.longitudes)

    def points_latlon(self) -> np.ndarray:
        return np.column_stack([self._lon_np, self._lat_np])

    @property
    def cfl_length_scale(self) -> float:
        return self.min_edge_length

    @property
    def cell_areas(self) -> torch.Tensor:
        """Barycentric 'Voronoi' areas (1/3 of each spherical triangle,
        L'Huilier excess), geodesic_grid.py:200-266."""
        return self._cell_areas


def _warn_if_underresolved(n_points: int, l_max: int):
    """Warn below MIN_POINTS_PER_BASIS points per (l, m>=0) mode,
    optimized_geodesic_sh.py:25-39."""
    n_basis = (l_max + 1) * (l_max + 2) // 2
    ratio = n_points / n_basis
    if ratio < MIN_POINTS_PER_BASIS:
        l_safe = int((np.sqrt(1.0 + 8.0 * n_points / MIN_POINTS_PER_BASIS) - 3.0) / 2.0)
        warnings.warn(
            f"Geodesic SH is under-resolved: {n_points} points for l_max={l_max} ({n_basis} basis functions, "
            f"{ratio:.1f} pts/basis < {MIN_POINTS_PER_BASIS:.0f}); round trips leak energy across modes. "
            f"Use l_max <= {l_safe} at this resolution, or a finer grid.", stacklevel=3)


class PointSetSphericalHarmonics:
    """Dense transform on arbitrary points, fast_geodesic_sh.py:8-111."""

    def __init__(self, latitudes, longitudes, l_max: int, weights=None, radius: float = 1.0, device=None):
        lat = latitudes.detach().cpu().numpy() if torch.is_tensor(latitudes) else np.asarray(latitudes, float)
        lon = longitudes.detach().cpu().numpy() if torch.is_tensor(longitudes) else np.asarray(longitudes, float)
        if lat.shape != lon.shape:
            raise AssertionError("Latitude and Longitude arrays must have the same shape.")
        if lat.ndim != 1:
            raise AssertionError("Input lat/lon must be 1D arrays.")
        w = None
        if weights is not None:
            w = weights.detach().cpu().numpy() if torch.is_tensor(weights) else np.asarray(weights, float)
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        self.l_max = int(l_max)
        self.n_points = lat.size
        self.n_basis = (self.l_max + 1) * (self.l_max + 2) // 2
        self.plan = Plan.points(lat, lon, w, self.l_max, radius, self.device)
        self.latitudes = torch.from_numpy(np.ascontiguousarray(lat, float)).to(self.device)
        self.longitudes = torch.from_numpy(np.ascontiguousarray(lon, float)).to(self.device)
        self.weights = (torch.full((self.n_points,), 4.0 * np.pi / self.n_points, dtype=torch.float64,
                                   device=self.device)
                        if w is None else torch.from_numpy(np.ascontiguousarray(w, float)).to(self.device))
        self.grid_shape = (self.n_points,)

    def transform(self, values) -> torch.Tensor:
        v = torch.as_tensor(values, dtype=torch.float64, device=self.device)
        if v.dim() > 1 and v.shape[-1] != self.n_points:
            v = v.reshape(-1)
        return analyze(self.plan.id, v)

    def inv_transform(self, coeffs) -> torch.Tensor:
        return synthesize(self.plan.id, torch.as_tensor(coeffs, device=self.device))

    inverse_transform = inv_transform


class GeodesicSphericalHarmonics:
    """Weight-aware geodesic wrapper, optimized_geodesic_sh.py:42-151.

    weights: "voronoi" (areas / R^2 renormalised to sum 4 pi), "uniform",
    None, or an explicit array.  "optimize" (host BVLS weight fitting) is
    not part of the GB300 path and raises.
    """

    def __init__(self, grid: GeodesicGridGeometry, l_max=None, cache_dir=None, weights="voronoi",
                 latitudes=None, longitudes=None):
        if l_max is None:
            raise ValueError("l_max is required.")
        self.grid = grid
        self.l_max = int(l_max)
        if grid is None:
            if latitudes is None or longitudes is None:
                raise ValueError("Provide either grid or latitudes/longitudes.")
            if isinstance(weights, str) and weights in ("optimize", "voronoi"):
                raise ValueError("weights='optimize' or 'voronoi' requires a grid.")
            _warn_if_underresolved(len(latitudes), self.l_max)
            w = None if (weights is None or weights == "uniform") else weights
            self.sh = PointSetSphericalHarmonics(latitudes, longitudes, self.l_max, weights=w)
        else:
            if latitudes is not None or longitudes is not None:
                raise ValueError("Provide either grid or latitudes/longitudes, not both.")
            _warn_if_underresolved(grid.n_points, self.l_max)
            w = None
            if isinstance(weights, str):
                mode = weights.lower()
                if mode == "voronoi":
                    a = grid.cell_areas / grid.radius ** 2          # optimized_geodesic_sh.py:127-133
                    w = a * (4.0 * np.pi) / torch.sum(a)
                elif mode == "optimize":
                    raise ValueError("weights='optimize' (host least-squares fitting) is not available on the "
                                     "GB300 path; use 'voronoi', 'uniform' or explicit weights")
                elif mode != "uniform":
                    raise ValueError(f"Unknown weights mode: {weights}")
            elif weights is not None:
                w = weights
            self.sh = PointSetSphericalHarmonics(grid._lat_np, grid._lon_np, self.l_max, weights=w,
                                                 radius=grid.radius, device=grid.device)
        self.weights = self.sh.weights
        self.plan = self.sh.plan
        self.latitudes = self.sh.latitudes
        self.longitudes = self.sh.longitudes
        self.n_points = self.sh.n_points

    def transform(self, values):
        return self.sh.transform(values)

    def inv_transform(self, coeffs):
        return self.sh.inv_transform(coeffs)

    inverse_transform = inv_transform
