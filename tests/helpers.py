"""Shared numeric helpers for the parity tests."""
import numpy as np


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def tri(c):
    """Zero the m > l storage slots (the layout leaves them unspecified)."""
    c = np.array(c, copy=True)
    L = c.shape[-1] - 1
    l = np.arange(L + 1)
    c[..., l[None, :] > l[:, None]] = 0
    return c
