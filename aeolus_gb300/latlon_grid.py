"""Gauss-Legendre lat-lon geometry and its transform on the GB300 path.

Mirrors src/planetary_sandbox/numerics/latlon_grid.py (same names, argument
meaning, layout and errors).  The transform is not a dense basis product:
it is a per-order Legendre contraction plus a longitude real FFT
(``csrc/legendre.cuh``, ``csrc/rows.cuh``), with Gauss nodes from an FP64
Newton iteration on the device.
"""
from __future__ import annotations

import warnings

import numpy as np
import torch

from .ops import Plan, analyze, synthesize


def _device(device):
    return torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())


class GaussLatLonGridGeometry:
    """Gauss-Legendre x uniform-longitude grid, latlon_grid.py:43-148.

    Rows run north -> south; per-point arrays are the C-order flattening of
    the (nlat, nlon) grid.  Arrays are float64 CUDA tensors.
    """

    def __init__(self, nlat: int, nlon: int, radius: float = 1.0, device=None):
        if nlat < 2 or nlon < 4:
            raise ValueError(
                f"GaussLatLonGridGeometry needs nlat >= 2 and nlon >= 4, got ({nlat}, {nlon})")
        self.nlat, self.nlon, self.radius = int(nlat), int(nlon), float(radius)
        self.device = _device(device)
        nodes = Plan.gauss(self.nlat, self.nlon, 0, self.radius, self.device)
        lat, w_gl = nodes.nodes()
        nodes.close()
        self._latitudes_np = lat
        self._longitudes_np = np.linspace(0.0, 2.0 * np.pi, self.nlon, endpoint=False)
        self._gl_weights = w_gl
        dev = self.device
        self._latitudes = torch.from_numpy(lat).to(dev)
        self._longitudes = torch.from_numpy(self._longitudes_np).to(dev)
        self._point_latitudes = self._latitudes.repeat_interleave(self.nlon)
        self._point_longitudes = self._longitudes.repeat(self.nlat)
        self.coslat = torch.cos(self._point_latitudes)
        self.sinlat = torch.sin(self._point_latitudes)
        w_point = np.repeat(w_gl, self.nlon) * (2.0 * np.pi / self.nlon)
        self.solid_angle_weights = torch.from_numpy(w_point).to(dev)

    latitudes = property(lambda self: self._latitudes)
    longitudes = property(lambda self: self._longitudes)
    point_latitudes = property(lambda self: self._point_latitudes)
    point_longitudes = property(lambda self: self._point_longitudes)

    @property
    def n_points(self) -> int:
        return self.nlat * self.nlon

    @property
    def grid_shape(self) -> tuple[int, int]:
        return (self.nlat, self.nlon)

    def points_latlon(self) -> np.ndarray:
        return np.column_stack([self._point_longitudes.cpu().numpy(), self._point_latitudes.cpu().numpy()])

    @property
    def cell_areas(self) -> torch.Tensor:
        return self.solid_angle_weights * self.radius ** 2

    @property
    def cfl_length_scale(self) -> float:
        """R * min meridional node spacing, latlon_grid.py:125-148."""
        colat = np.pi / 2.0 - self._latitudes_np
        return self.radius * float(np.min(np.abs(np.diff(colat))))


class GaussLatLonSphericalHarmonics:
    """Analysis/synthesis on a GaussLatLonGridGeometry, latlon_grid.py:151-199.

    ``transform`` / ``inv_transform`` accept leading batch dimensions; with
    none they behave exactly like the reference (flat (n_points,) fields,
    (L+1, L+1) complex coefficients).
    """

    def __init__(self, grid: GaussLatLonGridGeometry, l_max: int):
        if not isinstance(grid, GaussLatLonGridGeometry):
            raise ValueError(
                f"GaussLatLonSphericalHarmonics requires a GaussLatLonGridGeometry, got {type(grid).__name__}")
        self.grid = grid
        self.l_max = int(l_max)
        if grid.nlat < l_max + 1 or grid.nlon < 2 * l_max + 1:
            warnings.warn(
                f"Gauss lat-lon SH is under-resolved: ({grid.nlat}, {grid.nlon}) grid for l_max={l_max}. "
                f"Analysis is exact only for nlat >= {l_max + 1} and nlon >= {2 * l_max + 1}; "
                f"below that, round trips leak energy across modes.", stacklevel=2)
        self.plan = Plan.gauss(grid.nlat, grid.nlon, self.l_max, grid.radius, grid.device)
        self.weights = grid.solid_angle_weights
        self.n_points = grid.n_points
        self.latitudes = grid.point_latitudes
        self.longitudes = grid.point_longitudes
        self.grid_shape = (grid.n_points,)

    def transform(self, values) -> torch.Tensor:
        """Analysis: values (flat, (nlat, nlon), or batched) -> coefficients."""
        v = torch.as_tensor(values, dtype=torch.float64, device=self.grid.device)
        if v.dim() >= 2 and tuple(v.shape[-2:]) == (self.grid.nlat, self.grid.nlon):
            v = v.reshape(tuple(v.shape[:-2]) + (self.n_points,))
        return analyze(self.plan.id, v)

    def inv_transform(self, coeffs) -> torch.Tensor:
        """Synthesis: coefficients -> flat (n_points,) field(s)."""
        c = torch.as_tensor(coeffs, device=self.grid.device)
        return synthesize(self.plan.id, c)

    inverse_transform = inv_transform


def fine_dims(nlat: int, nlon: int, l_max: int) -> tuple[int, int]:
    """3/2-rule product grid, spherical_backend.py:201-203."""
    return max((3 * l_max) // 2 + 1, nlat), max(3 * l_max + 1, nlon)


__all__ = ["GaussLatLonGridGeometry", "GaussLatLonSphericalHarmonics", "fine_dims"]
