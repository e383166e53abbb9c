"""Backend seam: geometry + transform + product-space policy.

Mirrors src/planetary_sandbox/numerics/spherical_backend.py:43-241 (same
classes, modes, caching and "no silent fallback" errors).  Product spaces
hold GB300 transforms; the Gauss "fine" space is the 3/2-rule grid and is the
state transform itself when the rule gives back the state dimensions.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from dataclasses import dataclass
from typing import Any

import torch

from .geodesic_grid import GeodesicGridGeometry, GeodesicSphericalHarmonics
from .latlon_grid import GaussLatLonGridGeometry, GaussLatLonSphericalHarmonics, fine_dims

_COSLAT_FLOOR = 1e-8  # spherical_backend.py:72


@dataclass(frozen=True)
class ProductSpace:
    sh: Any
    coslat: torch.Tensor
    geometry: Any
    label: str


class SphericalGridBackend(ABC):
    def __init__(self, geometry, sh):
        self.geometry = geometry
        self.sh = sh
        self.l_max = sh.l_max
        self._product_spaces: dict[str, ProductSpace] = {}

    @abstractmethod
    def supported_product_quadratures(self) -> tuple[str, ...]:
        ...

    def product_space(self, mode: str) -> ProductSpace:
        if mode not in self.supported_product_quadratures():
            raise ValueError(
                f"product_quadrature must be one of {self.supported_product_quadratures()}, got {mode!r} "
                f"(backend {type(self).__name__}; no silent fallback)")
        if mode not in self._product_spaces:
            self._product_spaces[mode] = self._build_product_space(mode)
        return self._product_spaces[mode]

    @abstractmethod
    def _build_product_space(self, mode: str) -> ProductSpace:
        ...

    def describe(self, product_quadrature: str) -> dict:
        return {
            "backend": type(self).__name__,
            "grid": type(self.geometry).__name__,
            "state_sampling": self.product_space("coarse").label,
            "product_quadrature": product_quadrature,
            "product_sampling": self.product_space(product_quadrature).label,
            "transform": type(self.sh).__name__,
            "l_max": int(self.l_max),
        }

    def _coarse_coslat(self) -> torch.Tensor:
        coslat = getattr(self.geometry, "coslat", None)
        if coslat is None:
            coslat = torch.cos(torch.as_tensor(self.geometry.point_latitudes))
        return torch.clamp(coslat, min=_COSLAT_FLOOR)


class GeodesicBackend(SphericalGridBackend):
    """'fine' = resolution r+1 geodesic co-grid with Voronoi weights."""

    def __init__(self, geometry, sh):
        if not isinstance(geometry, GeodesicGridGeometry):
            raise ValueError(f"GeodesicBackend requires a GeodesicGridGeometry, got {type(geometry).__name__}")
        super().__init__(geometry, sh)

    def supported_product_quadratures(self):
        return ("coarse", "fine")

    def _build_product_space(self, mode):
        if mode == "coarse":
            return ProductSpace(self.sh, self._coarse_coslat(), None,
                                f"geodesic-res{self.geometry.resolution}-state")
        fine = GeodesicGridGeometry(self.geometry.resolution + 1, self.geometry.radius, self.geometry.device)
        fine_sh = GeodesicSphericalHarmonics(fine, self.l_max, weights="voronoi")
        return ProductSpace(fine_sh, torch.clamp(fine.coslat, min=_COSLAT_FLOOR), fine,
                            f"geodesic-res{fine.resolution}-voronoi")


class LatLonBackend(SphericalGridBackend):
    """'fine' = 3/2-rule Gauss product grid (exact for quadratic products)."""

    def __init__(self, geometry, sh):
        if not isinstance(geometry, GaussLatLonGridGeometry):
            raise ValueError(f"LatLonBackend requires a GaussLatLonGridGeometry, got {type(geometry).__name__}")
        super().__init__(geometry, sh)

    def supported_product_quadratures(self):
        return ("coarse", "fine")

    def _build_product_space(self, mode):
        g = self.geometry
        if mode == "coarse":
            return ProductSpace(self.sh, self._coarse_coslat(), None, f"latlon-gauss-{g.nlat}x{g.nlon}-state")
        nf, mf = fine_dims(g.nlat, g.nlon, self.l_max)
        if (nf, mf) == (g.nlat, g.nlon):
            # The 3/2 rule gives back the state grid: reuse its transform
            # (identical points and weights, so identical results).
            fine_geometry, fine_sh = g, self.sh
        else:
            fine_geometry = GaussLatLonGridGeometry(nf, mf, g.radius, g.device)
            fine_sh = GaussLatLonSphericalHarmonics(fine_geometry, self.l_max)
        return ProductSpace(fine_sh, torch.clamp(fine_geometry.coslat, min=_COSLAT_FLOOR), fine_geometry,
                            f"latlon-gauss-{nf}x{mf}-3/2rule")


class PointSetBackend(SphericalGridBackend):
    def supported_product_quadratures(self):
        return ("coarse",)

    def _build_product_space(self, mode):
        return ProductSpace(self.sh, self._coarse_coslat(), None, "point-set-state")


def make_backend(geometry, sh) -> SphericalGridBackend:
    if isinstance(geometry, GeodesicGridGeometry):
        return GeodesicBackend(geometry, sh)
    if isinstance(geometry, GaussLatLonGridGeometry):
        return LatLonBackend(geometry, sh)
    return PointSetBackend(geometry, sh)
