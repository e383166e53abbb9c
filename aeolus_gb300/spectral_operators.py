"""Spectral operators on the shared (L+1, L+1) complex layout.

Mirrors src/planetary_sandbox/numerics/spectral_operators.py:53-658.  The
diagonal / tridiagonal operators run as one elementwise kernel each
(``aeolus_spectral_op``); the pseudospectral Jacobian is one fused chain
(derivative coefficients -> synthesis -> product -> analysis -> 2/3 cut).
"""
from __future__ import annotations

import torch

from . import _lib
from .ops import Plan, jacobian, spectral_op, vector_curl_div, winds
from .spherical_backend import make_backend


class SpectralOperators:
    def __init__(self, sh, radius: float, grid=None, product_quadrature: str = "coarse", backend=None):
        self.sh = sh
        self.R = float(radius)
        self.l_max = sh.l_max
        self.grid = grid
        self.backend = backend if backend is not None else make_backend(grid, sh)
        self.product_quadrature = product_quadrature
        self._product_space = self.backend.product_space(product_quadrature)
        self.product_grid = self._product_space.geometry
        self.product_sh = self._product_space.sh if self._product_space.geometry is not None else None
        dev = getattr(sh, "weights").device
        l = torch.arange(self.l_max + 1, dtype=torch.float64, device=dev)
        self.lap_eigs = -l * (l + 1.0) / self.R ** 2          # :114
        self._vector_plan = None  # one-degree-extended analysis plan (:474-492), built on first use

    # -- diagonal / tridiagonal operators (one kernel each) --------------
    def laplacian_coeffs(self, coeffs):
        return spectral_op(_lib.SOP_LAPLACIAN, self.R, coeffs)

    def d_lambda_coeffs(self, coeffs):
        return spectral_op(_lib.SOP_D_LAMBDA, self.R, coeffs)

    def sin_theta_d_theta_coeffs(self, coeffs):
        return spectral_op(_lib.SOP_SIN_THETA_D_THETA, self.R, coeffs)

    def adjoint_sin_theta_d_theta_coeffs(self, coeffs):
        return spectral_op(_lib.SOP_ADJOINT_SIN_THETA_D_THETA, self.R, coeffs)

    def inv_laplacian(self, coeffs):
        """l = 0 mode divided by 1/R^2 (i.e. times R^2), :275-292."""
        return spectral_op(_lib.SOP_INV_LAPLACIAN, self.R, coeffs)

    def inv_d_lambda(self, coeffs):
        """(R / (i m)) a for m >= 1, zero at m = 0, :294-311."""
        m = torch.arange(self.l_max + 1, dtype=torch.float64, device=coeffs.device)
        inv = torch.zeros(self.l_max + 1, dtype=torch.complex128, device=coeffs.device)
        inv[1:] = 1.0 / (1j * m[1:] / self.R)
        return inv[None, :] * coeffs

    def _truncate_product(self, coeffs):
        return spectral_op(_lib.SOP_TRUNCATE, self.R, coeffs)

    def laplacian_field(self, coeffs):
        return self.sh.inv_transform(self.laplacian_coeffs(coeffs))

    def d_lambda_field(self, coeffs):
        return self.sh.inv_transform(self.d_lambda_coeffs(coeffs))

    def sin_theta_d_theta_field(self, coeffs):
        return self.sh.inv_transform(self.sin_theta_d_theta_coeffs(coeffs))

    # -- nonlinear ---------------------------------------------------------
    def jacobian_pseudospectral(self, a_lm, b_lm, dealias: bool = True, return_spectral: bool = False):
        """J(a, b) = (a_snt b_lam - a_lam b_snt) / cos^2 on the product space,
        :590-658.  The (dealias, return_spectral) = (True, True) form is one
        fused chain; the legacy grid-returning forms are composed from it."""
        ps = self._product_space
        sh_p = ps.sh
        if dealias:
            J_lm = jacobian(sh_p.plan.id, a_lm, b_lm)
            return J_lm if return_spectral else self.sh.inv_transform(J_lm)
        a_lam = sh_p.inv_transform(self.d_lambda_coeffs(a_lm))
        b_lam = sh_p.inv_transform(self.d_lambda_coeffs(b_lm))
        a_snt = sh_p.inv_transform(self.sin_theta_d_theta_coeffs(a_lm)) / self.R
        b_snt = sh_p.inv_transform(self.sin_theta_d_theta_coeffs(b_lm)) / self.R
        J_grid = (a_snt * b_lam - a_lam * b_snt) / ps.coslat ** 2
        if return_spectral:
            return sh_p.transform(J_grid)
        if sh_p is self.sh:
            return J_grid
        return self.sh.inv_transform(sh_p.transform(J_grid))

    # -- vector fields ---------------------------------------------------------
    def vector_curl_div_spectral(self, f_east, f_north, *, truncate: bool = True):
        """(curl_lm, div_lm) of a tangent field sampled on the product points by
        the weak form with one-degree-extended analyses, :399-492 (one analysis
        chain on the extended plan, one spectral kernel)."""
        plan = self._extended_plan()
        dev = plan.device
        fe = torch.as_tensor(f_east, dtype=torch.float64, device=dev)
        fn = torch.as_tensor(f_north, dtype=torch.float64, device=dev)
        out = vector_curl_div(plan.id, self.R, fe, fn, bool(truncate))
        return out[0], out[1]

    def vector_curl_div_roundtrip(self, f_east, f_north, *, truncate: bool = True):
        """Scalar round-trip curl/div of a tangent field on the product points
        (:336-397; the reference's own comparison pathway, not its production
        one): analyse each component, synthesize their derivatives, assemble
        div = (fu_lam - fv_snt)/cos - tan/R fv, curl = (fu_snt + fv_lam)/cos +
        tan/R fu from the round-tripped components, analyse (2/3 cut)."""
        ps = self._product_space
        sh_p, coslat = ps.sh, ps.coslat
        dev = sh_p.weights.device
        fe = torch.as_tensor(f_east, dtype=torch.float64, device=dev).reshape(-1)
        fn = torch.as_tensor(f_north, dtype=torch.float64, device=dev).reshape(-1)
        cl = coslat.reshape(-1)
        sinlat = torch.sin(torch.as_tensor(sh_p.latitudes, dtype=torch.float64, device=dev)).reshape(-1)
        fu_lm, fv_lm = sh_p.transform(fe), sh_p.transform(fn)
        lam = lambda c: sh_p.inv_transform(self.d_lambda_coeffs(c))  # noqa: E731
        snt = lambda c: sh_p.inv_transform(self.sin_theta_d_theta_coeffs(c)) / self.R  # noqa: E731
        fu_rt, fv_rt = sh_p.inv_transform(fu_lm), sh_p.inv_transform(fv_lm)
        tan_over_r = sinlat / (self.R * cl)
        div_g = (lam(fu_lm) - snt(fv_lm)) / cl - tan_over_r * fv_rt
        curl_g = (snt(fu_lm) + lam(fv_lm)) / cl + tan_over_r * fu_rt
        curl_lm, div_lm = sh_p.transform(curl_g), sh_p.transform(div_g)
        if truncate:
            curl_lm, div_lm = self._truncate_product(curl_lm), self._truncate_product(div_lm)
        return curl_lm, div_lm

    def _extended_plan(self):
        """The product points and weights with the basis extended to degree
        l_max + 1 (_vector_analysis_pieces, :474-492), in the product plan's
        precision mode."""
        plan = self._extended_plan_base()
        want = self._product_space.sh.plan.precision
        if plan.precision != want:
            plan.set_precision(want)
        return plan

    def _extended_plan_base(self):
        if self._vector_plan is None:
            from .latlon_grid import GaussLatLonSphericalHarmonics
            sh_p = self._product_space.sh
            if isinstance(sh_p, GaussLatLonSphericalHarmonics):
                g = sh_p.grid
                self._vector_plan = Plan.gauss(g.nlat, g.nlon, self.l_max + 1, g.radius, g.device)
            else:
                lat, lon, w = (x.detach().cpu().numpy() for x in (sh_p.latitudes, sh_p.longitudes, sh_p.weights))
                self._vector_plan = Plan.points(lat, lon, w, self.l_max + 1, self.R, sh_p.weights.device)
        return self._vector_plan

    def velocity_from_streamfunction(self, psi_lm):
        """(u, v) on the state sampling, |cos lat| < 1e-6 -> 0; :517-538."""
        uv = winds(self.sh.plan.id, self.R, psi_lm, None)
        return uv[0], uv[1]

    def grad_from_scalar(self, q_lm):
        """((1/(R cos)) q_lam, (1/R) q_phi) on the state sampling, :542-560."""
        coslat = torch.cos(self.sh.latitudes)
        q_lam = self.sh.inv_transform(self.d_lambda_coeffs(q_lm))
        gq = self.sh.inv_transform(self.sin_theta_d_theta_coeffs(q_lm))
        return q_lam / coslat, -gq / (self.R * coslat)

    def advect_scalar_by_streamfunction(self, psi_lm, q_lm, dealias: bool = True, return_spectral: bool = False):
        """u . grad(q) on the state sampling, :564-588."""
        u, v = self.velocity_from_streamfunction(psi_lm)
        dq_dx, dq_dy = self.grad_from_scalar(q_lm)
        adv = u * dq_dx + v * dq_dy
        if not (dealias or return_spectral):
            return adv
        adv_lm = self.sh.transform(adv)
        if dealias:
            adv_lm = self._truncate_product(adv_lm)
        return adv_lm if return_spectral else self.sh.inv_transform(adv_lm)


__all__ = ["SpectralOperators"]
