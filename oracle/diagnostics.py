"""Oracle conservation diagnostics (TEST INFRASTRUCTURE ONLY).

Restates src/planetary_sandbox/run/bve/diagnostics.py:52-124 and the
invariant sums of src/planetary_sandbox/run/swe/diagnostics.py:76-173.
"""
from __future__ import annotations

import math

import numpy as np


def mode_power(c):
    """Per-(l,m) power for the m>=0 layout, bve/diagnostics.py:52-58."""
    n_l, n_m = c.shape
    l_idx, m_idx = np.indices((n_l, n_m))
    p = np.where(m_idx == 0, c.real ** 2, 2.0 * np.abs(c) ** 2)
    return np.where(m_idx <= l_idx, p, 0.0)


def spectral_diagnostics(zeta, radius: float, omega: float) -> dict:
    """bve/diagnostics.py:61-97."""
    R = float(radius)
    L = zeta.shape[0] - 1
    l = np.arange(L + 1.0)
    P = mode_power(zeta)
    Z_l = 0.5 * R ** 2 * P.sum(axis=1)
    inv = np.zeros(L + 1)
    inv[1:] = 1.0 / (l[1:] * (l[1:] + 1.0))
    E_l = 0.5 * R ** 4 * inv * P.sum(axis=1)
    q = zeta.copy()
    q[1, 0] += 2.0 * omega * math.sqrt(4.0 * math.pi / 3.0)
    Z_abs = float(0.5 * R ** 2 * mode_power(q).sum())
    Z = float(Z_l.sum())
    cut = (2 * L) // 3
    return {
        "circulation": float(R ** 2 * math.sqrt(4.0 * math.pi) * zeta[0, 0].real),
        "energy": float(E_l.sum()),
        "enstrophy_rel": Z,
        "enstrophy_abs": Z_abs,
        "energy_l1": float(E_l[1]),
        "high_l_enstrophy_frac": float(Z_l[cut + 1:].sum()) / Z if Z > 0 else 0.0,
    }


def grid_diagnostics(zeta, sh, radius: float, omega: float) -> dict:
    """bve/diagnostics.py:100-124 (quadrature form)."""
    R = float(radius)
    w = sh.weights * R ** 2
    z = sh.inv_transform(zeta)
    f = 2.0 * omega * np.sin(sh.latitudes)
    L = zeta.shape[0] - 1
    l = np.arange(L + 1.0)
    psi = np.zeros_like(zeta)
    psi[1:, :] = zeta[1:, :] / (-l[1:] * (l[1:] + 1.0) / R ** 2)[:, None]
    p = sh.inv_transform(psi)
    return {
        "circulation": float(np.sum(z * w)),
        "energy": float(-0.5 * np.sum(p * z * w)),
        "enstrophy_rel": float(0.5 * np.sum(z ** 2 * w)),
        "enstrophy_abs": float(0.5 * np.sum((z + f) ** 2 * w)),
    }


def swe_invariants(model, coeffs) -> dict:
    """Mass (spectral), energy (quadrature), L2 norms; swe/diagnostics.py:76-173."""
    R = model.R
    sh = model.ops.sh
    u, v = model.wind_on_state_grid(coeffs)
    phi_total = model.phi0 + sh.inv_transform(coeffs[2])
    w = sh.weights * R ** 2
    ke = 0.5 * phi_total * (u ** 2 + v ** 2)
    pe = 0.5 * phi_total ** 2
    l2 = lambda c: float(np.sqrt(R ** 2 * mode_power(c).sum()))  # noqa: E731
    return {
        "total_mass": R ** 2 * (4.0 * math.pi * model.phi0
                                + math.sqrt(4.0 * math.pi) * float(coeffs[2][0, 0].real)),
        "total_energy": float(np.sum(w * (ke + pe))),
        "zeta_l2": l2(coeffs[0]),
        "delta_l2": l2(coeffs[1]),
        "phi_l2": l2(coeffs[2]),
    }
