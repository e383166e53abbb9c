"""Adjoints on the GPU: transposed transforms (dot-product identities),
tendency and RK4 vector-Jacobian products against central finite
differences of the forward kernels and of the CPU oracle, and the
checkpointed multi-step gradient of the SWE geopotential misfit.

Tolerances: transposes 1e-12 relative (exact up to rounding); gradients
1e-7 relative against central differences (eps = 1e-6 relative); split-
precision gradients 1e-6 relative L2 against the FP64 gradient.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from oracle import models as omodels

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.adjoint import bve_rk4_checkpointed, swe_rk4_checkpointed, weighted_phi_misfit
from aeolus_gb300.barotropic import BarotropicState, BarotropicVorticity
from aeolus_gb300.ops import (Plan, analyze, analyze_adjoint, bve_tendency_adjoint, swe_rk4_adjoint,
                              swe_tendency_adjoint, synthesize, synthesize_adjoint)
from aeolus_gb300.shallow_water import ShallowWaterModel

pytestmark = pytest.mark.gpu
DEV = "cuda"


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


def tri_mask(L):
    l = np.arange(L + 1)
    return l[None, :] <= l[:, None]


def rand_spec(rng, shape, L):
    a = rng.standard_normal(shape + (L + 1, L + 1)) + 1j * rng.standard_normal(shape + (L + 1, L + 1))
    return a * tri_mask(L)


def rdot(a, b):
    """Real inner product of complex (Re, Im) vectors or of real arrays."""
    a, b = np.asarray(a), np.asarray(b)
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        return float(np.sum(a.real * b.real + a.imag * b.imag))
    return float(np.sum(a * b))


def points_plan(L, n=900, seed=3):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1, 1, n)
    lat = np.arcsin(z)
    lon = rng.uniform(-math.pi, math.pi, n)
    w = rng.uniform(0.5, 1.5, n)
    w *= 4 * math.pi / w.sum()
    return Plan.points(lat, lon, w, L)


# --------------------------------------------------------------- transforms
@pytest.mark.parametrize("kind,nlat,nlon,L", [("gauss", 32, 64, 21), ("gauss", 23, 45, 15), ("gauss", 192, 384, 127),
                                              ("points", 0, 0, 12)])
@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_transform_transposes(kind, nlat, nlon, L, precision):
    """<S a, g> = <a, S^T g> and <A f, c> = <f, A^T c> (batched)."""
    if precision == "split" and (kind != "gauss" or nlat < 32):
        pytest.skip("split precision covers Gauss plans with FFT rows")
    p = Plan.gauss(nlat, nlon, L) if kind == "gauss" else points_plan(L)
    if precision == "split":
        p.set_precision(_lib.PREC_SPLIT_BF16)
    rng = np.random.default_rng(L)
    a = rand_spec(rng, (3,), L)
    c = rand_spec(rng, (3,), L)
    g = rng.standard_normal((3, p.n_points))
    f = rng.standard_normal((3, p.n_points))
    Sa, STg = N(synthesize(p.id, T(a))), N(synthesize_adjoint(p.id, T(g)))
    Af, ATc = N(analyze(p.id, T(f))), N(analyze_adjoint(p.id, T(c)))
    tol = 1e-12 if precision == "fp64" else 1e-11
    for b in range(3):
        lhs, rhs = rdot(Sa[b], g[b]), rdot(a[b], STg[b])
        assert abs(lhs - rhs) <= tol * (np.linalg.norm(Sa[b]) * np.linalg.norm(g[b])), (b, lhs, rhs)
        lhs, rhs = rdot(Af[b], c[b]), rdot(f[b], ATc[b])
        assert abs(lhs - rhs) <= tol * (np.linalg.norm(Af[b]) * np.linalg.norm(c[b])), (b, lhs, rhs)
    # m > l slots of the transposed synthesis are zero, Im of m = 0 too
    assert np.all(STg[:, ~tri_mask(L)] == 0) and np.all(STg[:, :, 0].imag == 0)


def test_autograd_through_transforms():
    p = Plan.gauss(32, 64, 21)
    rng = np.random.default_rng(0)
    a = T(rand_spec(rng, (2,), 21)).requires_grad_(True)
    tgt = T(rng.standard_normal((2, p.n_points)))
    loss = ((synthesize(p.id, a) - tgt) ** 2).sum()
    (ga,) = torch.autograd.grad(loss, a)
    g = N(2 * (synthesize(p.id, a.detach()) - tgt))
    np.testing.assert_allclose(N(ga), N(synthesize_adjoint(p.id, T(g))), rtol=0, atol=1e-12 * np.abs(N(ga)).max())
    f = T(rng.standard_normal((2, p.n_points))).requires_grad_(True)
    c = analyze(p.id, f)
    (gf,) = torch.autograd.grad((c.abs() ** 2).sum(), f)
    np.testing.assert_allclose(N(gf), N(analyze_adjoint(p.id, 2 * c.detach())), rtol=1e-12,
                               atol=1e-14 * np.abs(N(gf)).max())


# ---------------------------------------------------------------- tendencies
def _fd_dir(fun, y, d, eps):
    return (fun(y + eps * d) - fun(y - eps * d)) / (2 * eps)


def _check_vjp(fwd, vjp, y, kb, dirs, tol=1e-7):
    """<vjp(kb), d> vs <kb, (fwd(y + e d) - fwd(y - e d)) / 2e> per direction."""
    yb = N(vjp(T(y), T(kb)))
    ny = np.linalg.norm(y)
    for d in dirs:
        eps = 1e-6 * ny / np.linalg.norm(d)
        fd = rdot(kb, N(_fd_dir(lambda x: fwd(x), T(y), T(d), eps)))
        ad = rdot(yb, d)
        assert abs(ad - fd) <= tol * max(abs(fd), 1e-300) + 1e-14 * np.linalg.norm(yb) * np.linalg.norm(d), (ad, fd)


@pytest.mark.parametrize("grid", ["gauss", "gauss_fine", "geodesic"])
def test_bve_tendency_vjp_matches_fd(grid):
    if grid == "geodesic":
        planet = ae.make_planet("geodesic", resolution=3, l_max=10)
        L = 10
    else:
        L = 21 if grid == "gauss" else 15
        nlat, nlon = (32, 64) if grid == "gauss" else (16, 32)
        planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    model = BarotropicVorticity(planet, viscosity=1e5)
    rng = np.random.default_rng(1)
    z = np.stack([W.bve_vorticity(L, s) for s in range(2)])
    kb = rand_spec(rng, (2,), L)
    dirs = [rand_spec(rng, (2,), L) for _ in range(4)]
    pid = model._plan.id
    _check_vjp(lambda x: model.tendency(BarotropicState(x)),
               lambda y, k: bve_tendency_adjoint(pid, model.R, model.Omega, model.nu, y, k), z, kb, dirs)


@pytest.mark.parametrize("nlat,nlon,L", [(32, 64, 21), (16, 32, 15), (20, 30, 15)])
def test_swe_tendency_vjp_matches_fd(nlat, nlon, L):
    """Gauss grids with FFT rows, a distinct 3/2-rule product grid (16x32 ->
    23x46 products) and a direct-DFT row length."""
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    s, depth = W.member_states(L, 2, seed=5)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth, hyperdiffusion_nu4=1e14)
    rng = np.random.default_rng(2)
    kb = rand_spec(rng, (2, 3), L) * np.array([1e-5, 1e-5, 1.0])[None, :, None, None]
    dirs = [rand_spec(rng, (2, 3), L) * np.abs(s).max(axis=(-1, -2), keepdims=True) for _ in range(4)]
    pid = model._plan.id
    _check_vjp(model.tendency,
               lambda y, k: swe_tendency_adjoint(pid, model.R, model.Omega, model.gravity, model.mean_depth, model.nu4,
                                                 y, k), s, kb, dirs)


def test_swe_tendency_vjp_matches_oracle_fd():
    """The gradient is that of the reference's discrete tendency: central
    differences of the CPU oracle (numpy restatement) along two directions."""
    L, nlat, nlon = 21, 32, 64
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    s, depth = W.member_states(L, 1, seed=9)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    sh = oracle.GaussSH(nlat, nlon, L)
    ops = oracle.Operators(sh, W.EARTH_RADIUS, sh_p=sh)
    om = omodels.SWE(ops, W.EARTH_OMEGA, W.GRAVITY, depth)
    rng = np.random.default_rng(4)
    kb = rand_spec(rng, (3,), L) * np.array([1e-5, 1e-5, 1.0])[:, None, None]
    yb = N(swe_tendency_adjoint(model._plan.id, model.R, model.Omega, model.gravity, model.mean_depth, 0.0,
                                T(s), T(kb[None])))[0]
    for _ in range(2):
        d = rand_spec(rng, (3,), L) * np.abs(s[0]).max(axis=(-1, -2), keepdims=True)
        eps = 1e-6 * np.linalg.norm(s[0]) / np.linalg.norm(d)
        fd = rdot(kb, (om.tendency(s[0] + eps * d) - om.tendency(s[0] - eps * d)) / (2 * eps))
        assert abs(rdot(yb, d) - fd) <= 1e-7 * abs(fd)


# ----------------------------------------------------------------- RK4 steps
def test_swe_rk4_step_adjoint_matches_fd():
    L = 21
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L)
    s, depth = W.member_states(L, 2, seed=11)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    rng = np.random.default_rng(6)
    kb = rand_spec(rng, (2, 3), L) * np.array([1.0, 1.0, 1e-5])[None, :, None, None]
    dirs = [rand_spec(rng, (2, 3), L) * np.abs(s).max(axis=(-1, -2), keepdims=True) for _ in range(3)]
    pid, dt = model._plan.id, 600.0
    _check_vjp(lambda x: model.rk4(x, dt, 1, check=False),
               lambda y, k: swe_rk4_adjoint(pid, model.R, model.Omega, model.gravity, model.mean_depth, 0.0, y, k, dt),
               s, kb, dirs)


def test_bve_checkpointed_gradient_matches_fd():
    L, dt, nsteps = 21, 900.0, 7
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L)
    model = BarotropicVorticity(planet, viscosity=1e5)
    rng = np.random.default_rng(8)
    z0 = T(W.bve_vorticity(L, 3)[None])
    w = T(rand_spec(rng, (1,), L))

    def loss(z):
        return (torch.view_as_real(bve_rk4_checkpointed(model, z, dt, nsteps, every=3) * w.conj()).sum())

    z = z0.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(loss(z), z)
    for _ in range(3):
        d = T(rand_spec(rng, (1,), L)) * float(z0.abs().max())
        eps = 1e-6 * float(torch.linalg.vector_norm(z0)) / float(torch.linalg.vector_norm(d))
        fd = float((loss(z0 + eps * d) - loss(z0 - eps * d)) / (2 * eps))
        assert abs(rdot(N(g), N(d)) - fd) <= 1e-7 * abs(fd)


def _c5_setup(L=127, nlat=192, nlon=384, nsteps=48, precision="fp64"):
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    if precision == "split":
        planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    y0, depth = W.perturbed_williamson2(L, seed=0)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    yt, _ = W.perturbed_williamson2(L, seed=1)
    target = synthesize(model._state_plan.id, model.rk4(T(yt[None]), 240.0, nsteps, check=False)[:, 2])
    return model, T(y0[None]), target


@pytest.mark.parametrize("L,nlat,nlon,nsteps,ndirs", [(21, 32, 64, 12, 8), (127, 192, 384, 48, 32)])
def test_swe_misfit_gradient_matches_central_fd(L, nlat, nlon, nsteps, ndirs):
    """Gradient of the area-weighted final-geopotential misfit through
    `nsteps` RK4 steps (dt 240 s, checkpoints every 8 steps) against central
    differences (eps = 1e-6 relative) on `ndirs` random directions, all
    directions evaluated as one batch of 2 * ndirs members."""
    model, y0, target = _c5_setup(L, nlat, nlon, nsteps)
    y = y0.clone().requires_grad_(True)
    J = weighted_phi_misfit(model, swe_rk4_checkpointed(model, y, 240.0, nsteps, every=8), target).sum()
    (g,) = torch.autograd.grad(J, y)
    rng = np.random.default_rng(7)
    scale = np.abs(N(y0)).max(axis=(-1, -2), keepdims=True)
    D = np.concatenate([rand_spec(rng, (1, 3), L) * scale for _ in range(ndirs)])
    eps = 1e-6 * float(torch.linalg.vector_norm(y0)) / np.linalg.norm(D.reshape(ndirs, -1), axis=1)
    E = T(eps[:, None, None, None] * D)
    Y = torch.cat([y0 + E, y0 - E])
    Jp = weighted_phi_misfit(model, model.rk4(Y, 240.0, nsteps, check=False), target)
    fd = N((Jp[:ndirs] - Jp[ndirs:])) / (2 * eps)
    ad = np.array([rdot(N(g)[0], D[i]) for i in range(ndirs)])
    err = np.abs(ad - fd) / np.abs(fd)
    assert err.max() <= 1e-7, err


def test_swe_split_gradient_matches_fp64_gradient():
    """Split-precision forward + adjoint against the FP64 plain path at the
    headline grid (12 steps, checkpoints every 8)."""
    grads = {}
    for prec in ("fp64", "split"):
        model, y0, target = _c5_setup(nsteps=12, precision=prec)
        y = y0.clone().requires_grad_(True)
        J = weighted_phi_misfit(model, swe_rk4_checkpointed(model, y, 240.0, 12, every=8), target).sum()
        (grads[prec],) = torch.autograd.grad(J, y)
    a, b = N(grads["split"]), N(grads["fp64"])
    for f in range(3):
        rel = np.linalg.norm(a[0, f] - b[0, f]) / np.linalg.norm(b[0, f])
        assert rel < 1e-6, (f, rel)
