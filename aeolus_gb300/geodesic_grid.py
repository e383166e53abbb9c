"""Icosahedral geodesic point set and the point-set transforms.

Mirrors src/planetary_sandbox/numerics/geodesic_grid.py (geometry, point
order, Voronoi areas), numerics/fast_geodesic_sh.py
(``PointSetSphericalHarmonics``) and numerics/optimized_geodesic_sh.py
(``GeodesicSphericalHarmonics`` with "voronoi" / "uniform" / explicit
weights).  The geometry is built on the host with vectorised NumPy; the
transform is a dense real basis built and contracted on the device
(``csrc/points.cu``).
"""
from __future__ import annotations

import warnings

import numpy as np
import torch

from .ops import Plan, analyze, synthesize

_PHI = (1.0 + np.sqrt(5.0)) / 2.0
# Icosahedron, geodesic_grid.py:15-28 (the point order depends on it).
_ICO_V = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                   [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                   [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]]) / np.hypot(1, _PHI)
_ICO_F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                   [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                   [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                   [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])

MIN_POINTS_PER_BASIS = 6  # optimized_geodesic_sh.py:23


def _subdivide_once(verts: np.ndarray, faces: np.ndarray):
    """One midpoint refinement; new vertices numbered in order of first use
    by (face, edge 12 / 23 / 31), the order of geodesic_grid.py:116-131."""
    e = np.stack([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]], axis=1).reshape(-1, 2)
    key = np.sort(e, axis=1)
    code = key[:, 0].astype(np.int64) * (len(verts) + 1) + key[:, 1]
    uniq, first, inv = np.unique(code, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")          # first-appearance order
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    mid_id = len(verts) + rank[inv].reshape(-1, 3)      # m12, m23, m31 per face
    a, b = key[first[order], 0], key[first[order], 1]
    mid = (verts[a] + verts[b]) / 2.0
    mid /= np.linalg.norm(mid, axis=1)[:, None]
    v1, v2, v3 = faces[:, 0], faces[:, 1], faces[:, 2]
    m12, m23, m31 = mid_id[:, 0], mid_id[:, 1], mid_id[:, 2]
    nf = np.stack([np.stack([v1, m12, m31], 1), np.stack([v2, m23, m12], 1),
                   np.stack([v3, m31, m23], 1), np.stack([m12, m23, m31], 1)], axis=1).reshape(-1, 3)
    return np.concatenate([verts, mid]), nf


class GeodesicGridGeometry:
    """Icosahedral geodesic grid, geodesic_grid.py:11-266."""

    def __init__(self, resolution: int = 0, radius: float = 1.0, device=None):
        self.resolution = int(resolution)
        self.radius = float(radius)
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        c, s = np.cos(1e-2), np.sin(1e-2)                     # :37-38 rotation about x
        rot = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
        verts, faces = _ICO_V @ rot.T, _ICO_F.copy()
        for _ in range(self.resolution):
            verts, faces = _subdivide_once(verts, faces)
        self.points = self.radius * verts
        self.faces = faces.astype(np.int32)
        self.n_points = len(self.points)
        self.n_faces = len(self.faces)
        x, y, z = self.points[:, 0], self.points[:, 1], self.points[:, 2]
        self._lat_np = np.arctan2(z, np.hypot(x, y))            # cartesian_to_spherical.py
        self._lon_np = np.arctan2(y, x)
        edges = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        d = np.linalg.norm(self.points[edges[:, 0]] - self.points[edges[:, 1]], axis=1)
        self.min_edge_length = float(d[d > 0].min()) if np.any(d > 0) else 0.0
        dev = self.device
        self.latitudes = torch.from_numpy(self._lat_np).to(dev)
        self.longitudes = torch.from_numpy(self._lon_np).to(dev)
        self.sinlat = torch.sin(self.latitudes)
        self.coslat = torch.cos(self.latitudes)
        self._cell_areas = None

    point_latitudes = property(lambda self: self.latitudes)
    point_longitudes = property(lambda self: self.longitudes)

    def points_latlon(self) -> np.ndarray:
        return np.column_stack([self._lon_np, self._lat_np])

    @property
    def cfl_length_scale(self) -> float:
        return self.min_edge_length

    @property
    def cell_areas(self) -> torch.Tensor:
        """Barycentric 'Voronoi' areas: 1/3 of each spherical triangle
        (L'Huilier excess), geodesic_grid.py:200-266."""
        if self._cell_areas is None:
            self._cell_areas = torch.from_numpy(self.voronoi_areas_np()).to(self.device)
        return self._cell_areas

    def voronoi_areas_np(self) -> np.ndarray:
        u = self.points / np.linalg.norm(self.points, axis=1)[:, None]
        f = self.faces
        a, b, c = u[f[:, 0]], u[f[:, 1]], u[f[:, 2]]
        ang = lambda p, q: np.arccos(np.clip(np.einsum("ij,ij->i", p, q), -1.0, 1.0))  # noqa: E731
        sa, sb, sc = ang(b, c), ang(a, c), ang(a, b)
        s = 0.5 * (sa + sb + sc)
        t = np.sqrt(np.tan(s / 2) * np.tan((s - sa) / 2) * np.tan((s - sb) / 2) * np.tan((s - sc) / 2))
        area = 4.0 * np.arctan(t) * self.radius ** 2 / 3.0
        out = np.zeros(self.n_points)
        np.add.at(out, f.ravel(), np.repeat(area, 3))
        return out


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
                    a = grid.voronoi_areas_np() / grid.radius ** 2
                    w = a * (4.0 * np.pi) / np.sum(a)
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
