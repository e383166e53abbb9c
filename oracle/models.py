"""Oracle BVE / SWE tendencies and RK4 (TEST INFRASTRUCTURE ONLY).

Restates src/planetary_sandbox/physics/barotropic.py:14-167,
src/planetary_sandbox/physics/shallow_water.py:144-539 (flat bottom, as in
every configuration here), src/planetary_sandbox/run/engine.py:406-431 and
src/planetary_sandbox/run/bve/runner.py:211-216.
"""
from __future__ import annotations

import math

import numpy as np

WILLIAMSON_GRAVITY = 9.80616                    # shallow_water.py:95


def f_lm(lmax: int, omega: float) -> np.ndarray:
    """Spectral planetary vorticity, barotropic.py:59-61."""
    f = np.zeros((lmax + 1, lmax + 1), dtype=np.complex128)
    f[1, 0] = 2.0 * omega * math.sqrt(4.0 * math.pi / 3.0)
    return f


def bve_tendency(ops, zeta, omega: float, nu: float = 0.0, forcing=None):
    """dζ/dt = -J(ψ, ζ+f) + ν λ_l ζ, l=0 row pinned; barotropic.py:120-167."""
    L = ops.l_max
    lap = -np.arange(L + 1.0) * (np.arange(L + 1.0) + 1.0) / ops.R ** 2
    psi = np.zeros_like(zeta)
    psi[1:, :] = zeta[1:, :] / lap[1:, None]                 # :91
    eta = zeta + f_lm(L, omega)                               # :147
    adv = -ops.jacobian_pseudospectral(psi, eta)              # :153-155
    lap_b = lap.copy()
    lap_b[0] = 1.0 / ops.R ** 2                               # :66
    out = adv + nu * lap_b[:, None] * zeta                    # :158-161
    if forcing is not None:
        out = out + forcing
    out[0, :] = 0.0                                           # :165
    return out


def bve_rk4_step(ops, zeta, dt: float, omega: float, nu: float = 0.0):
    """run/bve/runner.py:211-216."""
    t = lambda y: bve_tendency(ops, y, omega, nu)  # noqa: E731
    k1 = t(zeta)
    k2 = t(zeta + 0.5 * dt * k1)
    k3 = t(zeta + 0.5 * dt * k2)
    k4 = t(zeta + dt * k3)
    return zeta + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)


class SWE:
    """Shallow-water model, shallow_water.py:144-418 (flat bottom, nu4 >= 0)."""

    def __init__(self, ops, omega: float, gravity: float, mean_depth: float,
                 nu4: float = 0.0, elevation_lm=None):
        self.ops = ops
        self.R = ops.R
        self.Omega = float(omega)
        self.gravity = float(gravity)
        self.mean_depth = float(mean_depth)
        self.phi0 = self.gravity * self.mean_depth
        self.nu4 = float(nu4)
        self.l_max = ops.l_max
        self.f_lm = f_lm(self.l_max, omega)
        l = np.arange(self.l_max + 1.0)
        self.lap_eigs = -l * (l + 1.0) / self.R ** 2
        # bottom topography, shallow_water.py:226-271: phi_s = g h_s and its
        # mean-removed anomaly enter as constant spectral terms
        self.phi_s = None
        if elevation_lm is not None and np.any(elevation_lm):
            self.phi_s = self.gravity * np.asarray(elevation_lm, complex)
            self.phi_s_anom = self.phi_s.copy()
            self.phi_s_anom[0, 0] = 0.0

    def _inv_lap(self, c):                                    # :277-281
        out = np.zeros_like(c)
        out[1:, :] = c[1:, :] / self.lap_eigs[1:, None]
        return out

    def _deriv(self, sh, c):                                  # :292-303
        o = self.ops
        return (sh.inv_transform(o.d_lambda_coeffs(c)),
                sh.inv_transform(o.sin_theta_d_theta_coeffs(c)) / self.R)

    def _wind(self, sh, coslat, psi, chi):                    # :305-319
        psi_lam, psi_snt = self._deriv(sh, psi)
        chi_lam, chi_snt = self._deriv(sh, chi)
        return (psi_snt + chi_lam) / coslat, (psi_lam - chi_snt) / coslat

    def wind_on_state_grid(self, coeffs):                     # :321-325
        sh = self.ops.sh
        coslat = np.maximum(np.cos(sh.latitudes), 1e-8)
        return self._wind(sh, coslat, self._inv_lap(coeffs[0]),
                          self._inv_lap(coeffs[1]))

    def tendency(self, coeffs):                               # :347-418
        o = self.ops
        zeta, delta, phi = coeffs[0], coeffs[1], coeffs[2]
        psi = self._inv_lap(zeta)
        chi = self._inv_lap(delta)
        eta = zeta + self.f_lm
        sh, coslat = o.sh_p, o.coslat_p
        u, v = self._wind(sh, coslat, psi, chi)
        eta_lam, eta_snt = self._deriv(sh, eta)
        phi_lam, phi_snt = self._deriv(sh, phi)
        eta_g = sh.inv_transform(eta)
        zeta_g = sh.inv_transform(zeta)
        delta_g = sh.inv_transform(delta)
        phi_g = sh.inv_transform(phi)
        zeta_dot_g = -((u * eta_lam - v * eta_snt) / coslat + eta_g * delta_g)
        curl_g = eta_g * zeta_g + (v * eta_lam + u * eta_snt) / coslat
        ke_g = 0.5 * (u * u + v * v)
        phi_dot_g = -((u * phi_lam - v * phi_snt) / coslat + phi_g * delta_g)
        zeta_dot = o.truncate(sh.transform(zeta_dot_g))
        curl_c = o.truncate(sh.transform(curl_g))
        ke_c = o.truncate(sh.transform(ke_g))
        phi_dot = o.truncate(sh.transform(phi_dot_g)) - self.phi0 * delta
        delta_dot = curl_c - self.lap_eigs[:, None] * (ke_c + phi)
        if self.phi_s is not None:                            # :397-401
            delta_dot = delta_dot - self.lap_eigs[:, None] * self.phi_s
        out = np.stack([zeta_dot, delta_dot, phi_dot])
        if self.nu4 > 0.0:
            out -= self.nu4 * (self.lap_eigs[None, :, None] ** 2) * coeffs
            if self.phi_s is not None:                        # :408-413
                out[2] -= self.nu4 * (self.lap_eigs[:, None] ** 2) * self.phi_s_anom
        out[:, 0, :] = 0.0
        return out

    def total_geopotential_extrema(self, coeffs):             # :428-454
        samplings = [self.ops.sh]
        if self.ops.sh_p is not self.ops.sh:
            samplings.append(self.ops.sh_p)
        lo, hi = math.inf, -math.inf
        for sh in samplings:
            g = sh.inv_transform(coeffs[2])
            lo, hi = min(lo, float(g.min())), max(hi, float(g.max()))
        return self.phi0 + lo, self.phi0 + hi

    def validate_state(self, coeffs):
        """Return the list of violated checks (shallow_water.py:494-539)."""
        bad = []
        if not np.isfinite(coeffs).all():
            return ["nonfinite"]
        for idx, name in enumerate(("zeta", "delta", "phi")):
            mono = abs(coeffs[idx, 0, 0])
            scale = float(np.linalg.norm(coeffs[idx]))
            if mono > 1e-10 * max(scale, 1e-30):
                bad.append(f"monopole_{name}")
        lo, _ = self.total_geopotential_extrema(coeffs)
        if not lo > 0.0:
            bad.append("thickness")
        return bad


def rk4_step_array(tendency, y, dt: float):
    """run/engine.py:406-431 (no stage validator)."""
    k1 = tendency(y)
    k2 = tendency(y + 0.5 * dt * k1)
    k3 = tendency(y + 0.5 * dt * k2)
    k4 = tendency(y + dt * k3)
    return y + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)


def williamson2(lmax: int, radius: float, omega: float, gravity: float = WILLIAMSON_GRAVITY,
                gh0: float = 2.94e4):
    """Williamson case 2 base state + mean depth.

    run/swe/initial_conditions.py:74-101 for the coefficients;
    mean depth (gh0 - C/3)/g as in tests/test_williamson2.py:65.
    """
    u0 = 2.0 * math.pi * radius / (12.0 * 86400.0)
    C = radius * omega * u0 + 0.5 * u0 * u0
    s = np.zeros((3, lmax + 1, lmax + 1), dtype=np.complex128)
    s[0, 1, 0] = (2.0 * u0 / radius) * math.sqrt(4.0 * math.pi / 3.0)
    s[2, 2, 0] = -(4.0 * C / 3.0) * math.sqrt(math.pi / 5.0)
    mean_depth = (gh0 - C / 3.0) / gravity
    return s, mean_depth
