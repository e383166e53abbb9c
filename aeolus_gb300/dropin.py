"""GB300 transforms behind the reference's own operator stack.

The reference (``planetary_sandbox``) reaches a spherical-harmonic transform
only through a duck-typed protocol -- ``transform(values)``,
``inv_transform(coeffs)`` / ``inverse_transform``, ``l_max``, ``weights``,
``latitudes``, ``longitudes`` (numerics/fast_geodesic_sh.py:68-111,
numerics/latlon_grid.py:151-199) -- and the backend seam --
``product_space(mode)``, ``supported_product_quadratures()``, ``describe()``
(numerics/spherical_backend.py:43-241).  Its ``SpectralOperators``, physics
models, diagnostics and runners are written against those two objects.  This
module provides both, backed by the GB300 plans, for the caller's own array
type, so that the reference's code runs unchanged on these kernels:

    grid = GaussLatLonGridGeometry(nlat, nlon, R)          # the reference's
    sh = GaussTransform(grid, l_max)                       # this module
    backend = LatLonBackend(grid, sh)                      # this module
    so = SpectralOperators(sh, R, grid, product_quadrature="fine",
                           backend=backend)                # the reference's
    model = ShallowWaterModel(planet, ...)                 # the reference's

Arrays: NumPy arrays are copied to the device and back around each call
(the reference under NumPy); CUDA arrays that speak DLPack (CuPy, torch) go
to the kernels zero-copy and the results come back as the caller's array
type.  There is no CPU path: the transforms run on the GPU in both cases.

Gauss nodes: the plan computes its own nodes and weights by an FP64 Newton
iteration on the device (latitudes within 1 ulp and weights within 6e-15
of 50-digit rules), while the reference's geometry takes them from
``numpy.polynomial.legendre.leggauss`` (latlon_grid.py:60), which is off by
up to ~4e-11 relative in the polar weights at nlat = 192.  ``node_offsets``
states the largest difference between the two for the geometry given.
"""
from __future__ import annotations

import importlib
import warnings
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from .ops import Plan, analyze, synthesize

_COSLAT_FLOOR = 1e-8  # spherical_backend.py:72


# ------------------------------------------------------------------ arrays
def _is_cuda_array(x) -> bool:
    dl = getattr(x, "__dlpack_device__", None)
    if dl is None:
        return False
    try:
        return int(dl()[0]) == 2  # kDLCUDA
    except Exception:
        return False


def _to_device(x, device: torch.device, dtype=None) -> torch.Tensor:
    """`x` as a tensor on `device` (zero-copy for CUDA arrays already there);
    dtype None keeps the array's own."""
    if isinstance(x, torch.Tensor):
        t = x
    elif _is_cuda_array(x):
        t = torch.from_dlpack(x)
    else:
        t = torch.as_tensor(np.asarray(x))
    return t.to(device=device, dtype=dtype or t.dtype)


def _like(t: torch.Tensor, like):
    """`t` as the caller's array type (NumPy, torch, or the DLPack module of
    a CUDA array such as CuPy)."""
    if isinstance(like, torch.Tensor):
        return t
    if _is_cuda_array(like):
        mod = importlib.import_module(type(like).__module__.split(".")[0])
        return mod.from_dlpack(t)
    return t.cpu().numpy()


def _host(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    if _is_cuda_array(x):
        return torch.from_dlpack(x).cpu().numpy()
    return np.asarray(x)


def _real_values(v: torch.Tensor) -> torch.Tensor:
    if torch.is_complex(v):
        if bool(torch.any(v.imag != 0)):
            raise ValueError("transform() analyses real fields; got values with a nonzero imaginary part")
        v = v.real
    return v


# ------------------------------------------------------------------ transforms
class _Transform:
    """The reference's transform protocol over one GB300 plan."""

    plan: Plan
    l_max: int
    n_points: int

    def _device_values(self, values) -> torch.Tensor:
        v = _real_values(_to_device(values, self.plan.device)).to(torch.float64)
        shape = getattr(self, "_grid2d", None)
        if shape is not None and v.dim() >= 2 and tuple(v.shape[-2:]) == shape:
            v = v.reshape(tuple(v.shape[:-2]) + (self.n_points,))
        return v

    def transform(self, values):
        """Analysis: point values (flat, or (nlat, nlon) on a Gauss grid; with
        leading batch dimensions) -> (L+1, L+1) complex coefficients."""
        return _like(analyze(self.plan.id, self._device_values(values)), values)

    def inv_transform(self, coeffs):
        """Synthesis: (L+1, L+1) complex coefficients (with leading batch
        dimensions) -> flat (n_points,) float64 field(s); Im(a_l0) and the
        m > l slots are ignored, as in the reference."""
        c = _to_device(coeffs, self.plan.device, torch.complex128)
        return _like(synthesize(self.plan.id, c), coeffs)

    def inverse_transform(self, coeffs):
        """Alias for inv_transform."""
        return self.inv_transform(coeffs)


class GaussTransform(_Transform):
    """In place of GaussLatLonSphericalHarmonics (latlon_grid.py:151-199): the
    per-order Legendre contraction plus longitude real FFT of a GB300 Gauss
    plan, on the caller's Gauss geometry (duck-typed: ``nlat``, ``nlon``,
    ``radius``, ``point_latitudes``, ``point_longitudes``,
    ``solid_angle_weights``).  ``plan`` may share an existing plan of the
    same grid and degree."""

    def __init__(self, grid, l_max: int, device=None, plan: Plan | None = None):
        self.grid = grid
        self.l_max = int(l_max)
        nlat, nlon = int(grid.nlat), int(grid.nlon)
        if nlat < self.l_max + 1 or nlon < 2 * self.l_max + 1:
            warnings.warn(
                f"Gauss lat-lon SH is under-resolved: ({nlat}, {nlon}) grid for l_max={self.l_max}. "
                f"Analysis is exact only for nlat >= {self.l_max + 1} and nlon >= {2 * self.l_max + 1}; "
                f"below that, round trips leak energy across modes.", stacklevel=2)
        if plan is None:
            plan = Plan.gauss(nlat, nlon, self.l_max, float(grid.radius), device)
        elif (plan.nlat, plan.nlon, plan.lmax) != (nlat, nlon, self.l_max):
            raise ValueError("GaussTransform: the shared plan is for another grid or degree")
        self.plan = plan
        self.n_points = nlat * nlon
        self._grid2d = (nlat, nlon)
        self.weights = grid.solid_angle_weights
        self.latitudes = grid.point_latitudes
        self.longitudes = grid.point_longitudes

    @property
    def node_offsets(self) -> dict:
        """Largest differences between the plan's Gauss nodes/weights and the
        geometry's (latitude in radians; weights relative)."""
        lat, w = self.plan.nodes()
        nlat, nlon = self._grid2d
        glat = _host(self.grid.point_latitudes).reshape(nlat, nlon)[:, 0]
        gw = _host(self.grid.solid_angle_weights).reshape(nlat, nlon)[:, 0] / (2.0 * np.pi / nlon)
        return {"max_abs_latitude": float(np.max(np.abs(lat - glat))),
                "max_rel_weight": float(np.max(np.abs(w - gw) / np.abs(gw)))}


class PointSetTransform(_Transform):
    """In place of PointSetSphericalHarmonics (fast_geodesic_sh.py:8-111) and
    of GeodesicSphericalHarmonics (optimized_geodesic_sh.py:42-151, whose
    Voronoi weights the caller passes): the basis product of a GB300 point-
    set plan over the caller's points and quadrature weights."""

    def __init__(self, latitudes, longitudes, l_max: int, weights=None, device=None):
        lat, lon = _host(latitudes).astype(np.float64), _host(longitudes).astype(np.float64)
        w = None if weights is None else _host(weights).astype(np.float64)
        self.l_max = int(l_max)
        self.plan = Plan.points(lat, lon, w, self.l_max, device=device)
        self.n_points = int(lat.size)
        self.latitudes, self.longitudes = latitudes, longitudes
        self.weights = weights if weights is not None else np.full(lat.size, 4.0 * np.pi / lat.size)


# ------------------------------------------------------------------ backend seam
@dataclass(frozen=True)
class ProductSpace:
    """Same fields as the reference's ProductSpace (spherical_backend.py:43-69)."""
    sh: Any
    coslat: Any
    geometry: Any
    label: str


def _floor_coslat(coslat):
    return coslat.clip(_COSLAT_FLOOR, None)


class LatLonBackend:
    """In place of the reference's LatLonBackend (spherical_backend.py:170-211),
    with GaussTransform product spaces: "coarse" is the state sampling,
    "fine" the 3/2-rule Gauss grid (nlat >= 3L/2 + 1, nlon >= 3L + 1).  The
    fine geometry is built with the state geometry's own class; when the rule
    gives back the state dimensions the fine transform is a distinct object
    sharing the state transform's plan (the reference builds a second,
    identical transform there)."""

    def __init__(self, geometry, sh: GaussTransform):
        for attr in ("nlat", "nlon", "radius"):
            if not hasattr(geometry, attr):
                raise ValueError(f"LatLonBackend requires a Gauss lat-lon geometry, got {type(geometry).__name__}")
        self.geometry = geometry
        self.sh = sh
        self.l_max = sh.l_max
        self._product_spaces: dict[str, ProductSpace] = {}

    def supported_product_quadratures(self) -> tuple[str, ...]:
        return ("coarse", "fine")

    def product_space(self, mode: str) -> ProductSpace:
        if mode not in self.supported_product_quadratures():
            raise ValueError(
                f"product_quadrature must be one of {self.supported_product_quadratures()}, got {mode!r} "
                f"(backend {type(self).__name__}; no silent fallback)")
        if mode not in self._product_spaces:
            self._product_spaces[mode] = self._build_product_space(mode)
        return self._product_spaces[mode]

    def _build_product_space(self, mode: str) -> ProductSpace:
        g = self.geometry
        if mode == "coarse":
            coslat = getattr(g, "coslat", None)
            if coslat is None:
                lat = g.point_latitudes
                coslat = _like(torch.cos(_to_device(lat, self.sh.plan.device, torch.float64)), lat)
            return ProductSpace(sh=self.sh, coslat=_floor_coslat(coslat), geometry=None,
                                label=f"latlon-gauss-{g.nlat}x{g.nlon}-state")
        nlat_f = max((3 * self.l_max) // 2 + 1, g.nlat)
        nlon_f = max(3 * self.l_max + 1, g.nlon)
        fine_geometry = type(g)(nlat_f, nlon_f, g.radius)
        same = (nlat_f, nlon_f) == (g.nlat, g.nlon)
        fine_sh = GaussTransform(fine_geometry, self.l_max, device=self.sh.plan.device,
                                 plan=self.sh.plan if same else None)
        return ProductSpace(sh=fine_sh, coslat=_floor_coslat(fine_geometry.coslat), geometry=fine_geometry,
                            label=f"latlon-gauss-{nlat_f}x{nlon_f}-3/2rule")

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


__all__ = ["GaussTransform", "PointSetTransform", "LatLonBackend", "ProductSpace"]
