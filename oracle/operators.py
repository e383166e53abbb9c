"""Oracle spectral operators (TEST INFRASTRUCTURE ONLY).

Restates src/planetary_sandbox/numerics/spectral_operators.py on NumPy
arrays in the shared dense (L+1, L+1) complex layout (axis 0 = l, axis 1 = m).
"""
from __future__ import annotations

import numpy as np


class Operators:
    """Diagonal / tridiagonal spectral operators, spectral_operators.py:53-334.

    ``sh`` is the state transform; ``sh_p``/``coslat_p`` the product space
    (spherical_backend.py:43-72): pointwise products are formed there.
    """

    def __init__(self, sh, radius: float, sh_p=None, coslat_p=None):
        self.sh = sh
        self.R = float(radius)
        self.l_max = L = sh.l_max
        self.sh_p = sh if sh_p is None else sh_p
        if coslat_p is None:
            coslat_p = np.cos(self.sh_p.latitudes)
        # spherical_backend.py:72,129 -- clamp away from zero.
        self.coslat_p = np.maximum(coslat_p, 1e-8)
        l = np.arange(L + 1, dtype=np.float64)
        m = np.arange(L + 1, dtype=np.float64)[None, :]
        self.lap_eigs = -l * (l + 1.0) / self.R ** 2            # :114
        self.im_m_over_R = 1j * m / self.R                      # :117 (m=0 -> 0)
        self.C_plus, self.C_minus = self._c_pm()

    def _c_pm(self):
        """sinθ∂θ coupling, spectral_operators.py:135-176 (C+[L,:] = 0)."""
        L = self.l_max
        Lb = np.broadcast_to(np.arange(L + 1.0)[:, None], (L + 1, L + 1))
        Mb = np.broadcast_to(np.arange(L + 1.0)[None, :], (L + 1, L + 1))
        valid = Mb <= Lb
        cp_ = Lb * np.sqrt(np.maximum((Lb + 1) ** 2 - Mb ** 2, 0.0)
                           / np.maximum((2 * Lb + 1) * (2 * Lb + 3), 1.0))
        cm_ = -(Lb + 1) * np.sqrt(np.maximum(Lb ** 2 - Mb ** 2, 0.0)
                                  / np.maximum((2 * Lb - 1) * (2 * Lb + 1), 1.0))
        cp_ = np.where(valid, cp_, 0.0)
        cm_ = np.where(valid, cm_, 0.0)
        cp_[L, :] = 0.0
        cm_[0, :] = 0.0
        return cp_, cm_

    def laplacian_coeffs(self, c):                              # :213-218
        return self.lap_eigs[:, None] * c

    def d_lambda_coeffs(self, c):                               # :220-226
        return self.im_m_over_R * c

    def sin_theta_d_theta_coeffs(self, c):                      # :228-241
        g = np.zeros_like(c, dtype=np.complex128)
        g[1:, :] += self.C_plus[:-1, :] * c[:-1, :]
        g[:-1, :] += self.C_minus[1:, :] * c[1:, :]
        return g

    def adjoint_sin_theta_d_theta_coeffs(self, c):              # :243-270
        g = np.zeros_like(c, dtype=np.complex128)
        g[:-1, :] += self.C_plus[:-1, :] * c[1:, :]
        g[1:, :] += self.C_minus[1:, :] * c[:-1, :]
        return g

    def inv_laplacian(self, c):                                 # :275-292 (l=0 * R^2)
        inv = self.lap_eigs.copy()
        inv[0] = 1.0 / self.R ** 2
        return c / inv[:, None]

    def inv_laplacian_zero(self, c):
        """Helmholtz inverse with l=0 zeroed, barotropic.py:91, shallow_water.py:277-281."""
        out = np.zeros_like(c)
        out[1:, :] = c[1:, :] / self.lap_eigs[1:, None]
        return out

    def truncate(self, c):
        """2/3 rule on rows AND columns, spectral_operators.py:329-334."""
        cut = (2 * self.l_max) // 3
        c[cut + 1:, :] = 0.0
        c[:, cut + 1:] = 0.0
        return c

    def jacobian_pseudospectral(self, a_lm, b_lm):
        """J(a,b) analysed on the product space + 2/3 cut, :590-658
        (dealias=True, return_spectral=True)."""
        sp = self.sh_p
        a_lam = sp.inv_transform(self.d_lambda_coeffs(a_lm))
        b_lam = sp.inv_transform(self.d_lambda_coeffs(b_lm))
        a_snt = sp.inv_transform(self.sin_theta_d_theta_coeffs(a_lm)) / self.R
        b_snt = sp.inv_transform(self.sin_theta_d_theta_coeffs(b_lm)) / self.R
        J = (a_snt * b_lam - a_lam * b_snt) / self.coslat_p ** 2
        return self.truncate(sp.transform(J))

    def vector_curl_div_spectral(self, f_east, f_north, sh_ext, truncate: bool = True):
        """Weak-form curl/div of a tangent field on the product points,
        spectral_operators.py:399-492: one-degree-extended half-metric
        analyses a = A(F_east/cos), b = A(F_north/cos) (``sh_ext``: the
        product points and weights with l_max + 1), then
        div = (i m/R) a + S^T b / R, curl = (i m/R) b - S^T a / R with the
        unclipped C+ at l = L reading the extended degree (:474-492)."""
        L = self.l_max
        n = L + 1
        a = sh_ext.transform(np.asarray(f_east) / self.coslat_p)
        b = sh_ext.transform(np.asarray(f_north) / self.coslat_p)
        Lb = np.broadcast_to(np.arange(n, dtype=np.float64)[:, None], (n, n))
        Mb = np.broadcast_to(np.arange(n, dtype=np.float64)[None, :], (n, n))
        c_plus_true = Lb * np.sqrt(np.maximum((Lb + 1.0) ** 2 - Mb ** 2, 0.0)
                                   / np.maximum((2.0 * Lb + 1.0) * (2.0 * Lb + 3.0), 1.0))
        c_plus_true = np.where(Mb <= Lb, c_plus_true, 0.0)

        def adjoint_ext(c_ext):
            out = c_plus_true * c_ext[1:n + 1, :n]
            out[1:, :] += self.C_minus[1:, :] * c_ext[:n - 1, :n]
            return out

        div = self.d_lambda_coeffs(a[:n, :n]) + adjoint_ext(b) / self.R
        curl = self.d_lambda_coeffs(b[:n, :n]) - adjoint_ext(a) / self.R
        if truncate:
            self.truncate(curl)
            self.truncate(div)
        return curl, div

    def velocity_from_streamfunction(self, psi_lm):
        """Winds on the state sampling, spectral_operators.py:517-538."""
        coslat = np.cos(self.sh.latitudes)
        safe = np.where(np.abs(coslat) < 1e-6, np.nan, coslat)
        lam = self.sh.inv_transform(self.d_lambda_coeffs(psi_lm))
        gpsi = self.sh.inv_transform(self.sin_theta_d_theta_coeffs(psi_lm))
        u = np.nan_to_num(gpsi / (self.R * safe), nan=0.0)
        v = np.nan_to_num(lam / safe, nan=0.0)
        return u, v
