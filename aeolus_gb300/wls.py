"""Weighted least-squares analysis on a point set.

The drop-in analysis is the reference's quadrature a = Y^H W f
(fast_geodesic_sh.py:68-87).  When the weights are not an exact quadrature
for degree 2 l_max (coarse or irregular point sets) the coefficients that
best fit the samples in the weighted norm solve the normal equations
S^T W S a = S^T W f, S the synthesis.  With the adjoint identity
S^T (W g) = s_m A(g) (A the quadrature analysis, s_0 = 1, s_m = 2; see
``aeolus_synthesize_adjoint``) this is  s A(S a) = s A(f): a symmetric
positive definite system on the m <= l coefficients (Im of m = 0 excluded),
close to s I whenever the quadrature is good, so preconditioned conjugate
gradients with the preconditioner s converge in a few iterations.  Every
product runs on the plan's kernels (FP64 or split precision).
"""
from __future__ import annotations

import torch

from .ops import analyze, synthesize


def _dot(x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """Real inner product per member over the (L+1)^2 slots."""
    return (x.real * y.real + x.imag * y.imag).sum(dim=(-2, -1))


def wls_analysis(plan, values: torch.Tensor, iters: int = 30, rtol: float = 1e-13):
    """Weighted least-squares coefficients of ``values`` ([..., n_points]).

    Returns (coefficients [..., L+1, L+1], iterations used, final relative
    residual of the normal equations per member)."""
    L = plan.lmax
    lead = tuple(values.shape[:-1])
    f = values.reshape(-1, plan.n_points).to(torch.float64)
    dev = f.device
    l = torch.arange(L + 1, device=dev)
    keep = (l[None, :] <= l[:, None]).to(torch.float64)
    s = torch.full((L + 1, L + 1), 2.0, dtype=torch.float64, device=dev)
    s[:, 0] = 1.0
    s = s * keep
    inv_s = torch.where(s > 0, 1.0 / s.clamp_min(1e-300), torch.zeros_like(s))

    def clean(a):  # m > l slots and Im(a_l0) are not unknowns
        a = a * keep
        return torch.complex(a.real, torch.cat([torch.zeros_like(a.imag[..., :1]), a.imag[..., 1:]], dim=-1))

    def M(a):
        return clean(s * analyze(plan.id, synthesize(plan.id, a)))

    b = clean(s * analyze(plan.id, f))
    x = clean(analyze(plan.id, f))            # the quadrature analysis as the first guess
    r = b - M(x)
    z = r * inv_s
    p = z
    rz = _dot(r, z)
    bn = torch.sqrt(_dot(b, b)).clamp_min(1e-300)
    res = torch.sqrt(_dot(r, r)) / bn
    it = 0
    while it < iters and bool((res > rtol).any()):
        q = M(p)
        alpha = rz / _dot(p, q).clamp_min(1e-300)
        x = x + alpha[:, None, None] * p
        r = r - alpha[:, None, None] * q
        res = torch.sqrt(_dot(r, r)) / bn
        z = r * inv_s
        rz_new = _dot(r, z)
        p = z + (rz_new / rz.clamp_min(1e-300))[:, None, None] * p
        rz = rz_new
        it += 1
    return x.reshape(lead + (L + 1, L + 1)), it, res
