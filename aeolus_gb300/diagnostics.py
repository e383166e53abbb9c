"""Conservation diagnostics on the device.

``spectral_diagnostics`` mirrors src/planetary_sandbox/run/bve/diagnostics.py:61-97
(one reduction kernel per call, deterministic order); ``grid_diagnostics``
mirrors :100-124 using the GB300 synthesis.
"""
from __future__ import annotations



import torch

from .ops import bve_spectral_diagnostics

_KEYS = ("circulation", "energy", "enstrophy_rel", "enstrophy_abs", "energy_l1", "high_l_enstrophy_frac")


def spectral_diagnostics(zeta_lm: torch.Tensor, radius: float, omega: float) -> dict:
    out = bve_spectral_diagnostics(float(radius), float(omega), zeta_lm)
    vals = out.reshape(-1, 6)[0].tolist() if out.dim() > 1 else out.tolist()
    return dict(zip(_KEYS, vals))


def grid_diagnostics(zeta_lm: torch.Tensor, sh, radius: float, omega: float, latitudes=None) -> dict:
    R = float(radius)
    w = sh.weights * R ** 2
    zeta = sh.inv_transform(zeta_lm)
    lat = sh.latitudes if latitudes is None else torch.as_tensor(latitudes, device=zeta.device)
    f = 2.0 * omega * torch.sin(lat)
    L = zeta_lm.shape[-1] - 1
    l = torch.arange(L + 1, dtype=torch.float64, device=zeta.device)
    psi_lm = torch.zeros_like(zeta_lm)
    lam = -l * (l + 1.0) / R ** 2
    psi_lm[1:, :] = zeta_lm[1:, :] / lam[1:, None]
    psi = sh.inv_transform(psi_lm)
    return {
        "circulation": float(torch.sum(zeta * w)),
        "energy": float(-0.5 * torch.sum(psi * zeta * w)),
        "enstrophy_rel": float(0.5 * torch.sum(zeta ** 2 * w)),
        "enstrophy_abs": float(0.5 * torch.sum((zeta + f) ** 2 * w)),
    }


