"""Oracle spherical-harmonic transforms (TEST INFRASTRUCTURE ONLY).

Two equivalent restatements of the reference transform
(src/planetary_sandbox/numerics/fast_geodesic_sh.py:8-111):

* ``PointSetSH`` -- the reference algorithm itself: a dense complex basis
  matrix ``Y[n_points, (L+1)(L+2)/2]`` with analysis ``a = Y^H (w*f)``
  scattered into the dense ``(L+1, L+1)`` layout (:68-87) and synthesis
  ``f = 2 Re(Y a) - Re(Y a|m=0)`` (:89-107).  Used for small sizes and as
  the timed CPU baseline.
* ``GaussSH`` -- the same sums on a Gauss grid, factored as a Legendre sum
  per zonal wavenumber plus a longitude DFT (``numpy.fft``), so the oracle
  reaches 192x384 / l_max=127 in seconds.  Checked against ``PointSetSH``.
"""
from __future__ import annotations

import numpy as np

FOUR_PI = 4.0 * np.pi


def n_coeff(lmax: int) -> int:
    """Number of (l, m>=0) modes, fast_geodesic_sh.py:47."""
    return (lmax + 1) * (lmax + 2) // 2


def gauss_latlon(nlat: int, nlon: int):
    """Gauss-Legendre x uniform-longitude geometry, latlon_grid.py:59-83.

    Returns (lat[nlat], lon[nlon], w_gl[nlat], w_point[nlat*nlon]); rows run
    north -> south, longitudes start at 0 with no seam duplicate, and the
    per-point solid-angle weights sum to 4*pi.
    """
    x, w_gl = np.polynomial.legendre.leggauss(nlat)
    order = np.argsort(-x)
    x, w_gl = x[order], w_gl[order]
    colat = np.arccos(x)
    lat = np.pi / 2.0 - colat
    lon = np.linspace(0.0, 2.0 * np.pi, nlon, endpoint=False)
    w_point = np.repeat(w_gl, nlon) * (2.0 * np.pi / nlon)
    return lat, lon, w_gl, w_point


def fine_dims(nlat: int, nlon: int, lmax: int):
    """3/2-rule product grid, spherical_backend.py:201-203."""
    return max((3 * lmax) // 2 + 1, nlat), max(3 * lmax + 1, nlon)


def legendre_table(x, s, lmax: int):
    """Orthonormal associated Legendre functions with Condon-Shortley phase.

    Same functions as sh_matrix.cu:31-60 (P_m^m seed with (-1)^m, norm
    sqrt((2l+1)/4pi (l-m)!/(l+m)!)), evaluated with the stable
    fully-normalised recurrence
        Pbar_mm     = -sqrt((2m+1)/(2m)) s Pbar_{m-1,m-1},  Pbar_00 = 1/sqrt(4pi)
        Pbar_{m+1,m} = sqrt(2m+3) x Pbar_mm
        Pbar_lm     = a_lm (x Pbar_{l-1,m} - Pbar_{l-2,m} / a_{l-1,m}),
        a_lm = sqrt((4l^2-1)/(l^2-m^2)).
    x = cos(colatitude), s = sin(colatitude) >= 0.  Returns a list over m of
    arrays shaped (lmax+1-m, npts).
    """
    x = np.asarray(x, dtype=np.float64)
    s = np.asarray(s, dtype=np.float64)
    out = []
    pmm = np.full(x.shape, 1.0 / np.sqrt(FOUR_PI))
    for m in range(lmax + 1):
        if m > 0:
            pmm = -np.sqrt((2.0 * m + 1.0) / (2.0 * m)) * s * pmm
        col = np.empty((lmax + 1 - m,) + x.shape)
        col[0] = pmm
        if m < lmax:
            col[1] = np.sqrt(2.0 * m + 3.0) * x * pmm
        for l in range(m + 2, lmax + 1):
            a = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            col[l - m] = a * (x * col[l - m - 1] - b * col[l - m - 2])
        out.append(col)
    return out


def dense_basis(lat, lon, lmax: int) -> np.ndarray:
    """Y[n, k], k = l(l+1)/2 + m (sh_matrix.cu:7-76 layout and convention)."""
    lat = np.asarray(lat, dtype=np.float64)
    lon = np.asarray(lon, dtype=np.float64)
    P = legendre_table(np.sin(lat), np.cos(lat), lmax)
    Y = np.empty((lat.size, n_coeff(lmax)), dtype=np.complex128)
    for m in range(lmax + 1):
        e = np.exp(1j * m * lon)
        for l in range(m, lmax + 1):
            Y[:, l * (l + 1) // 2 + m] = P[m][l - m] * e
    return Y


def lm_indices(lmax: int):
    """Flat-basis (l, m) index lists, fast_geodesic_sh.py:58-66."""
    ls, ms = [], []
    for l in range(lmax + 1):
        for m in range(l + 1):
            ls.append(l)
            ms.append(m)
    return np.array(ls), np.array(ms)


class PointSetSH:
    """Dense-basis transform on arbitrary points, fast_geodesic_sh.py:8-111."""

    def __init__(self, lat, lon, lmax: int, weights=None, basis=None):
        self.l_max = int(lmax)
        self.latitudes = np.ascontiguousarray(lat, dtype=np.float64)
        self.longitudes = np.ascontiguousarray(lon, dtype=np.float64)
        self.n_points = self.latitudes.size
        if weights is None:  # :35-37 uniform default
            self.weights = np.full(self.n_points, FOUR_PI / self.n_points)
        else:
            self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self.Y_matrix = (dense_basis(self.latitudes, self.longitudes, lmax)
                         if basis is None else basis)
        self.l_idx, self.m_idx = lm_indices(lmax)

    def transform(self, values) -> np.ndarray:
        """Analysis, fast_geodesic_sh.py:68-87."""
        v = np.asarray(values, dtype=np.float64).ravel()
        flat = self.Y_matrix.conj().T @ (v * self.weights)
        out = np.zeros((self.l_max + 1, self.l_max + 1), dtype=np.complex128)
        out[self.l_idx, self.m_idx] = flat
        return out

    def inv_transform(self, coeffs) -> np.ndarray:
        """Synthesis, fast_geodesic_sh.py:89-107 (Im a_l0 is discarded)."""
        flat = np.asarray(coeffs)[self.l_idx, self.m_idx]
        term = self.Y_matrix @ flat
        term0 = self.Y_matrix @ (flat * (self.m_idx == 0))
        return 2.0 * term.real - term0.real

    inverse_transform = inv_transform


class GaussSH:
    """Gauss-grid transform factored as per-m Legendre sums + longitude DFT.

    Mathematically identical to ``PointSetSH`` on the points of
    ``gauss_latlon(nlat, nlon)`` with the tensor-product weights
    (latlon_grid.py:151-199): Y_lm(j, k) = Pbar_lm(x_j) e^{i m lon_k}.
    """

    def __init__(self, nlat: int, nlon: int, lmax: int):
        self.nlat, self.nlon, self.l_max = int(nlat), int(nlon), int(lmax)
        lat, lon, w_gl, w_point = gauss_latlon(nlat, nlon)
        self.lat, self.lon, self.w_gl = lat, lon, w_gl
        self.weights = w_point
        self.latitudes = np.repeat(lat, nlon)
        self.longitudes = np.tile(lon, nlat)
        self.P = legendre_table(np.sin(lat), np.cos(lat), lmax)
        # e^{i m lon_k} for every m <= L (exact even when m >= nlon/2).
        self._E = np.exp(1j * np.outer(np.arange(lmax + 1), lon))

    def inv_transform(self, coeffs) -> np.ndarray:
        a = np.asarray(coeffs)
        L = self.l_max
        F = np.empty((L + 1, self.nlat), dtype=np.complex128)
        for m in range(L + 1):
            F[m] = a[m:, m] @ self.P[m]
        F[0] = F[0].real
        # f[j,k] = Re F_0 + 2 sum_{m>=1} Re(F_m e^{i m lon_k})
        g = 2.0 * (F.T @ self._E).real - F[0].real[:, None]
        return g.ravel()

    def transform(self, values) -> np.ndarray:
        f = np.asarray(values, dtype=np.float64).reshape(self.nlat, self.nlon)
        G = (f @ self._E.conj().T) * (self.w_gl[:, None] * (2.0 * np.pi / self.nlon))
        L = self.l_max
        out = np.zeros((L + 1, L + 1), dtype=np.complex128)
        for m in range(L + 1):
            out[m:, m] = self.P[m] @ G[:, m]
        return out

    inverse_transform = inv_transform
