"""Oracle dry hydrostatic primitive-equation tendency (TEST INFRASTRUCTURE ONLY).

Restates src/planetary_sandbox/physics/sigma_coordinate.py:43-400 (Lorenz
sigma grid, Simmons-Burridge hydrostatics, column continuity, energy-
conserving omega/p, centred vertical advection) and the tendency of
src/planetary_sandbox/physics/primitive_equations.py:482-753 on top of the
oracle transforms.  State rows are [zeta_1..K, delta_1..K, T_1..K, ln p_s].
"""
from __future__ import annotations

import math

import numpy as np

from .models import f_lm

R_DRY = 287.04      # primitive_equations.py:49
CP_DRY = 1004.64


class Sigma:
    """Interfaces sigma_{k+1/2}, top (0) to bottom (1); sigma_coordinate.py:43-149."""

    def __init__(self, interfaces):
        s = [float(x) for x in interfaces]
        if s[0] != 0.0 or s[-1] != 1.0 or any(b <= a for a, b in zip(s, s[1:])):
            raise ValueError("sigma interfaces must rise strictly from exactly 0 to exactly 1")
        self.s = s
        self.K = len(s) - 1
        self.dsig = [s[k + 1] - s[k] for k in range(self.K)]
        self.beta = [math.inf] + [math.log(s[k + 1] / s[k]) for k in range(1, self.K)]
        self.alpha = [math.log(2.0)] + [1.0 - (s[k] / self.dsig[k]) * self.beta[k] for k in range(1, self.K)]

    def hydrostatic(self, T, phi_s, r):
        """Full-level geopotential, :164-209 (linear: grid or spectral T)."""
        K = self.K
        below = [None] * K
        below[K - 1] = T[K - 1] * 0.0 + phi_s
        for k in range(K - 1, 0, -1):
            below[k - 1] = below[k] + (r * self.beta[k]) * T[k]
        return np.stack([below[k] + (r * self.alpha[k]) * T[k] for k in range(K)])

    def columns(self, G, A):
        """dlnps/dt, interface sigma_dot and omega/p, :212-253, :373-398."""
        K = self.K
        w = np.stack([self.dsig[k] * G[k] for k in range(K)])
        part = np.cumsum(w, axis=0)
        total = part[K - 1]
        sd = np.zeros((K + 1,) + G.shape[1:])
        for k in range(1, K):
            sd[k] = self.s[k] * total - part[k - 1]
        sd[K] = total - total
        wp = np.empty_like(G)
        wp[0] = A[0] - self.alpha[0] * G[0]
        for k in range(1, K):
            wp[k] = A[k] - (self.beta[k] / self.dsig[k]) * part[k - 1] - self.alpha[k] * G[k]
        return -w.sum(axis=0), sd, wp

    def vadv(self, sd, X):
        """Centred (sigma_dot dX/dsigma)_k, :280-305."""
        K = self.K
        out = np.zeros_like(X)
        for k in range(K):
            acc = None
            if k < K - 1:
                acc = sd[k + 1] * (X[k + 1] - X[k])
            if k > 0:
                up = sd[k] * (X[k] - X[k - 1])
                acc = up if acc is None else acc + up
            if acc is not None:
                out[k] = acc / (2.0 * self.dsig[k])
        return out


class PE:
    """primitive_equations.py:164-753 (explicit, full T, no hyperdiffusion)."""

    def __init__(self, ops, sigma: Sigma, omega: float, sh_ext, phi_s_lm=None,
                 r_dry: float = R_DRY, cp_dry: float = CP_DRY):
        self.ops, self.sig, self.sh_ext = ops, sigma, sh_ext
        self.R = ops.R
        self.L = ops.l_max
        self.r, self.kappa = float(r_dry), float(r_dry) / float(cp_dry)
        n = self.L + 1
        self.phi_s = np.zeros((n, n), complex) if phi_s_lm is None else np.asarray(phi_s_lm, complex)
        self.f_lm = f_lm(self.L, omega)
        l = np.arange(n, dtype=float)
        self.lap = -l * (l + 1.0) / self.R ** 2

    def _inv_lap(self, c):
        out = np.zeros_like(c)
        out[1:, :] = c[1:, :] / self.lap[1:, None]
        return out

    def _deriv(self, c):
        o, sp = self.ops, self.ops.sh_p
        return sp.inv_transform(o.d_lambda_coeffs(c)), sp.inv_transform(o.sin_theta_d_theta_coeffs(c)) / self.R

    def tendency(self, coeffs):
        o, sp, sg = self.ops, self.ops.sh_p, self.sig
        K, cosl = sg.K, o.coslat_p
        zeta, delta, temp, lnps = coeffs[:K], coeffs[K:2 * K], coeffs[2 * K:3 * K], coeffs[3 * K]
        lp_lam, lp_snt = self._deriv(lnps)
        u, v, zg, dg, tg, adv = ([] for _ in range(6))
        for k in range(K):                                        # :531-548
            psi_lam, psi_snt = self._deriv(self._inv_lap(zeta[k]))
            chi_lam, chi_snt = self._deriv(self._inv_lap(delta[k]))
            u.append((psi_snt + chi_lam) / cosl)
            v.append((psi_lam - chi_snt) / cosl)
            zg.append(sp.inv_transform(zeta[k]))
            dg.append(sp.inv_transform(delta[k]))
            tg.append(sp.inv_transform(temp[k]))
            adv.append((u[k] * lp_lam - v[k] * lp_snt) / cosl)
        u, v, zg, dg, tg, A = map(np.stack, (u, v, zg, dg, tg, adv))
        G = dg + A
        dlnps, sd, wp = sg.columns(G, A)
        phi_sg = sp.inv_transform(self.phi_s)
        sdU, sdV, sdT = sg.vadv(sd, u), sg.vadv(sd, v), sg.vadv(sd, tg)
        gu, gv = lp_lam / cosl, -lp_snt / cosl
        t_dot = []
        for k in range(K):                                        # :596-635
            t_lam, t_snt = self._deriv(temp[k])
            a = (u[k] * t_lam - v[k] * t_snt) / cosl
            t_dot.append(o.truncate(sp.transform(-a - sdT[k] + self.kappa * tg[k] * wp[k])))
        lnps_dot = o.truncate(sp.transform(dlnps))
        phi_lm = sg.hydrostatic(temp, self.phi_s, self.r)         # :691-693 (spectral T)
        z_dot, d_dot = [], []
        for k in range(K):                                        # :695-724
            eta = zeta[k] + self.f_lm
            e_lam, e_snt = self._deriv(eta)
            eg = sp.inv_transform(eta)
            div_ev = (u[k] * e_lam - v[k] * e_snt) / cosl + eg * dg[k]
            curl_ev = eg * zg[k] + (v[k] * e_lam + u[k] * e_snt) / cosl
            rt = self.r * tg[k]
            curl_z, div_z = o.vector_curl_div_spectral(sdU[k] + rt * gu, sdV[k] + rt * gv, self.sh_ext,
                                                       truncate=False)
            ke = o.truncate(sp.transform(0.5 * (u[k] * u[k] + v[k] * v[k])))
            z_dot.append(o.truncate(sp.transform(-div_ev) - curl_z))
            d_dot.append(o.truncate(sp.transform(curl_ev) - div_z) - self.lap[:, None] * (ke + phi_lm[k]))
        z_dot, d_dot = np.stack(z_dot), np.stack(d_dot)
        z_dot[:, 0, :] = 0.0
        d_dot[:, 0, :] = 0.0
        return np.concatenate([z_dot, d_dot, np.stack(t_dot), lnps_dot[None]], axis=0)
