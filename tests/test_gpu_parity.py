"""GPU parity of the sm_103a path against the reference golden vectors and
the CPU oracle, through the public API (C ABI underneath).

Tolerances: 1e-12 relative L2 for every float64 transform, tendency and RK4
result (the plain-FP64 drop-in bar); diagnostics to 1e-12 relative.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from oracle import models as omodels
from helpers import rel_l2, tri

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.ops import Plan, analyze, spectral_op, synthesize
from aeolus_gb300.barotropic import BarotropicVorticity, BarotropicState, rk4_step
from aeolus_gb300.shallow_water import ShallowWaterModel, ShallowWaterState, ShallowWaterStateError
from aeolus_gb300.diagnostics import spectral_diagnostics, grid_diagnostics

pytestmark = pytest.mark.gpu
TOL = 1e-12
DEV = "cuda"


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


def oracle_ops(nlat, nlon, L, R=W.EARTH_RADIUS):
    sh = oracle.GaussSH(nlat, nlon, L)
    nf, mf = oracle.fine_dims(nlat, nlon, L)
    sh_p = sh if (nf, mf) == (nlat, nlon) else oracle.GaussSH(nf, mf, L)
    return oracle.Operators(sh, R, sh_p=sh_p)


# ------------------------------------------------------------- transforms
@pytest.mark.parametrize("nlat", [2, 3, 16, 23, 32, 64, 96, 128, 160, 192])
def test_gauss_nodes_match_exact_rule(golden, nlat):
    """Device Newton nodes/weights vs 50-digit rules (tests/golden/make_gauss_exact.py).

    numpy.leggauss, the reference's node source (latlon_grid.py:60), is
    itself off by up to 4e-11 relative in the polar weights at nlat=192, so
    it is only checked loosely."""
    ex = golden("gauss_exact")
    p = Plan.gauss(nlat, 4 * nlat + 4, 1)
    lat, w = p.nodes()
    np.testing.assert_allclose(lat, ex[f"lat_{nlat}"], rtol=0, atol=5e-16)
    np.testing.assert_allclose(w, ex[f"w_{nlat}"], rtol=1e-14, atol=0)
    olat, _, ow, _ = oracle.gauss_latlon(nlat, 8)
    np.testing.assert_allclose(lat, olat, rtol=0, atol=5e-15)
    np.testing.assert_allclose(w, ow, rtol=1e-10, atol=0)
    assert abs(w.sum() - 2.0) < 1e-14


def test_bve_golden_transform(golden):
    g = golden("bve_gauss32x64_L21")
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=21)
    sh = planet.sh
    np.testing.assert_allclose(N(planet.grid.latitudes), g["lat"], rtol=0, atol=5e-15)
    np.testing.assert_allclose(N(sh.weights), g["weights"], rtol=1e-12)
    grid = sh.inv_transform(T(g["zeta"]))
    assert rel_l2(N(grid), g["grid"]) < TOL
    back = sh.transform(T(g["grid"]))
    assert rel_l2(N(back), g["roundtrip"]) < TOL


@pytest.mark.parametrize("nlat,nlon,L", [(32, 64, 21), (23, 46, 15), (16, 32, 15), (24, 48, 10), (17, 40, 12),
                                         (128, 256, 85), (160, 320, 106), (192, 384, 127), (20, 30, 15)])
def test_transforms_match_oracle(nlat, nlon, L):
    """FFT lengths 2^k, 2^k*3, 2^k*5 and the direct-DFT fallbacks (23, 15,
    nlon < 2L+2), odd nlat, batched."""
    rng = np.random.default_rng(nlat * 1000 + L)
    osh = oracle.GaussSH(nlat, nlon, L)
    p = Plan.gauss(nlat, nlon, L)
    a = np.stack([W.random_spectrum(rng, L, -1.5, 1.0, zero_monopole=False) for _ in range(3)])
    a[:, L // 2, 0] += 0.3j          # Im a_l0 must be ignored
    f = rng.standard_normal((3, nlat * nlon))
    g = N(synthesize(p.id, T(a)))
    c = N(analyze(p.id, T(f)))
    for b in range(3):
        assert rel_l2(g[b], osh.inv_transform(a[b])) < TOL
        assert rel_l2(tri(c[b]), osh.transform(f[b])) < TOL
        assert np.all(c[b][~W.triangle_mask(L)] == 0)


def test_roundtrip_l127_and_single_mode():
    p = Plan.gauss(192, 384, 127)
    rng = np.random.default_rng(5)
    a = W.random_spectrum(rng, 127, -1.5, 1.0, zero_monopole=False)
    back = N(analyze(p.id, synthesize(p.id, T(a))))
    assert rel_l2(back, a) < 1e-13
    d = np.zeros((128, 128), complex)
    d[127, 127] = 1.0 - 0.5j
    back = N(analyze(p.id, synthesize(p.id, T(d))))
    assert abs(back[127, 127] - d[127, 127]) < 1e-12 and np.abs(back - d).max() < 1e-12
    ones = torch.ones(192 * 384, dtype=torch.float64, device=DEV)
    a00 = N(analyze(p.id, ones))[0, 0]
    assert abs(a00 - math.sqrt(4 * math.pi)) / math.sqrt(4 * math.pi) < 1e-13


def test_empty_batch_and_bad_inputs():
    p = Plan.gauss(16, 32, 7)
    assert synthesize(p.id, torch.zeros((0, 8, 8), dtype=torch.complex128, device=DEV)).shape == (0, 512)
    with pytest.raises(ValueError):
        synthesize(p.id, torch.zeros((8, 9), dtype=torch.complex128, device=DEV))
    with pytest.raises(ValueError):
        analyze(p.id, torch.zeros(100, dtype=torch.float64, device=DEV))
    with pytest.raises(ValueError):
        synthesize(p.id, torch.zeros((8, 8), dtype=torch.complex128))  # CPU tensor: no fallback


# ------------------------------------------------------------- operators
def test_spectral_ops_match_oracle():
    L, R = 30, W.EARTH_RADIUS
    rng = np.random.default_rng(9)
    a = np.stack([W.random_spectrum(rng, L, -1.0, 1.0, zero_monopole=False) for _ in range(2)])
    sh = oracle.GaussSH(32, 64, L)
    ops = oracle.Operators(sh, R)
    cases = [(_lib.SOP_LAPLACIAN, ops.laplacian_coeffs), (_lib.SOP_INV_LAPLACIAN, ops.inv_laplacian),
             (_lib.SOP_INV_LAPLACIAN_ZERO, ops.inv_laplacian_zero), (_lib.SOP_D_LAMBDA, ops.d_lambda_coeffs),
             (_lib.SOP_SIN_THETA_D_THETA, ops.sin_theta_d_theta_coeffs),
             (_lib.SOP_ADJOINT_SIN_THETA_D_THETA, ops.adjoint_sin_theta_d_theta_coeffs),
             (_lib.SOP_TRUNCATE, lambda c: ops.truncate(c.copy()))]
    for op, ref in cases:
        out = N(spectral_op(op, R, T(a)))
        for b in range(2):
            assert rel_l2(out[b], tri(ref(a[b]))) < 1e-15, op


def test_jacobian_and_winds_match_oracle():
    L, R = 21, W.EARTH_RADIUS
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L)
    ops = oracle_ops(32, 64, L)
    rng = np.random.default_rng(4)
    a = W.random_spectrum(rng, L, -1.5, 1e6)
    b = W.random_spectrum(rng, L, -1.5, 1e-5)
    J = N(planet.so.jacobian_pseudospectral(T(a), T(b), dealias=True, return_spectral=True))
    assert rel_l2(J, ops.jacobian_pseudospectral(a, b)) < TOL
    u, v = planet.so.velocity_from_streamfunction(T(a))
    uo, vo = ops.velocity_from_streamfunction(a)
    assert rel_l2(N(u), uo) < TOL and rel_l2(N(v), vo) < TOL


def test_solid_body_jacobian():
    """J(psi_sb, Y_l^m) = i m omega Y_l^m (tests/test_spectral_operators.py:53-70)."""
    L, R = 21, W.EARTH_RADIUS
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L)
    omega = 1e-5
    psi = np.zeros((L + 1, L + 1), complex)
    psi[1, 0] = -omega * R ** 2 * math.sqrt(4 * math.pi / 3)   # psi = -omega R^2 sin(lat)
    for l, m in [(3, 2), (10, 7), (14, 1)]:
        q = np.zeros_like(psi)
        q[l, m] = 1.0
        J = N(planet.so.jacobian_pseudospectral(T(psi), T(q), return_spectral=True))
        expect = np.zeros_like(psi)
        expect[l, m] = 1j * m * omega
        assert np.abs(J - expect).max() < 1e-12 * max(m * omega, 1e-30) * 10


# ------------------------------------------------------------------ BVE
@pytest.mark.parametrize("name", ["bve_gauss32x64_L21", "bve_gauss16x32_L15_fine23x46"])
def test_bve_golden(golden, name):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    model = BarotropicVorticity(planet, viscosity=float(g["nu"]))
    z = T(g["zeta"])
    tend = model.tendency(BarotropicState(z))
    assert rel_l2(N(tend), g["tendency"]) < TOL
    step = rk4_step(model, BarotropicState(z), 0.0, float(g["dt"])).coeffs
    assert rel_l2(N(step), g["rk4"]) < TOL
    d1 = spectral_diagnostics(step, float(g["radius"]), float(g["omega"]))
    for k, v in zip(list(g["spec_keys"]), g["spec1"]):
        assert d1[k] == pytest.approx(v, rel=1e-10, abs=1e-300), k
    dg = grid_diagnostics(z, planet.sh, float(g["radius"]), float(g["omega"]))
    for k, v in zip(list(g["grid_keys"]), g["grid0"]):
        assert dg[k] == pytest.approx(v, rel=1e-11, abs=1e-3), k


def test_bve_batched_rk4_multi_step_matches_oracle():
    L, dt = 42, 900.0
    planet = ae.make_planet("latlon", nlat=64, nlon=128, l_max=L)
    ops = oracle_ops(64, 128, L)
    model = BarotropicVorticity(planet, viscosity=1e5)
    z0 = np.stack([W.bve_vorticity(L, s) for s in range(3)])
    y = N(model.rk4(T(z0), dt, 3))
    for b in range(3):
        ref = z0[b]
        for _ in range(3):
            ref = omodels.bve_rk4_step(ops, ref, dt, W.EARTH_OMEGA, 1e5)
        assert rel_l2(y[b], ref) < TOL


# ------------------------------------------------------------------ SWE
@pytest.mark.parametrize("name", ["swe_gauss16x32_L15_fine23x46", "swe_gauss32x64_L21", "swe_gauss128x256_L85"])
def test_swe_golden(golden, name):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    model = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    s = T(g["state"])
    assert rel_l2(N(model.tendency(s)), g["tendency"]) < TOL
    u, v = model.wind_on_state_grid(ShallowWaterState(s))
    assert rel_l2(N(u), g["u"]) < TOL and rel_l2(N(v), g["v"]) < TOL
    np.testing.assert_allclose(model.total_geopotential_extrema(ShallowWaterState(s)), g["phi_extrema"], rtol=1e-13)
    y = model.rk4(s, float(g["dt"]), int(g["steps"]))
    assert rel_l2(N(y), g["rk4"]) < TOL


def test_swe_l127_tendency_and_step_match_oracle():
    """The headline grid (192x384, l_max=127): the reference basis underflows
    there, so the pin is the oracle's stable recurrence."""
    L = 127
    planet = ae.make_planet("latlon", nlat=192, nlon=384, l_max=L)
    s0, depth = W.perturbed_williamson2(L, seed=21)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    om = omodels.SWE(oracle_ops(192, 384, L), W.EARTH_OMEGA, W.GRAVITY, depth)
    assert rel_l2(N(model.tendency(T(s0))), om.tendency(s0)) < TOL
    y = N(model.rk4(T(s0), 240.0, 1))
    assert rel_l2(y, omodels.rk4_step_array(om.tendency, s0, 240.0)) < TOL


def test_swe_fused_rk4_equals_composed_rk4():
    """model.rk4 (fused stages) == engine.rk4_step_array over model.tendency."""
    from aeolus_gb300.engine import rk4_step_array
    L = 21
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L)
    s, depth = W.member_states(L, 4, seed=3)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    y1 = model.rk4(T(s), 300.0, 2)
    y2 = T(s)
    for _ in range(2):
        y2 = rk4_step_array(model.tendency, y2, 0.0, 300.0)
    assert rel_l2(N(y1), N(y2)) < 1e-14


def test_williamson2_one_day_steady():
    """tests/test_williamson2.py:176-206 bounds: 1 day, 32x64, l_max=15."""
    L, R, om = 15, W.EARTH_RADIUS, 7.29212e-5
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=L, omega=om)
    s0, depth = W.williamson2(L, R, om)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    t0 = model.tendency(T(s0))
    u0 = 2 * math.pi * R / (12 * 86400.0)
    eta_amp = 2 * u0 / R + 2 * om
    assert float(t0[0].abs().max()) <= 1e-13 * (2 * u0 / R) * (u0 / R)
    assert float(t0[1].abs().max()) <= 1e-12 * (2 * u0 * eta_amp / R)
    assert float(t0[2].abs().max()) <= 1e-13 * model.phi0 * (2 * u0 / R)
    inv0 = model.invariants(ShallowWaterState(T(s0)))
    y = model.rk4(T(s0), 1440.0, 60)
    y_n = N(y)
    assert np.linalg.norm(y_n[0] - s0[0]) / np.linalg.norm(s0[0]) <= 1e-12
    assert np.linalg.norm(y_n[2] - s0[2]) / np.linalg.norm(s0[2]) <= 1e-12
    assert np.linalg.norm(y_n[1]) / np.linalg.norm(s0[0]) <= 1e-12
    inv1 = model.invariants(ShallowWaterState(y))
    assert abs(inv1["total_energy"] - inv0["total_energy"]) <= 1e-12 * inv0["total_energy"]
    assert inv1["total_mass"] == inv0["total_mass"]
    assert y_n[2, 0, 0] == 0


def test_swe_invariants_match_oracle(golden):
    g = golden("swe_gauss32x64_L21")
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=21)
    model = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    om = omodels.SWE(oracle_ops(32, 64, 21), float(g["omega"]), float(g["gravity"]), float(g["mean_depth"]))
    ref = oracle.diagnostics.swe_invariants(om, g["state"])
    got = model.invariants(ShallowWaterState(T(g["state"])))
    for k in ref:
        assert got[k] == pytest.approx(ref[k], rel=1e-12), k


def test_state_validation_faults_injected_on_host():
    """NaN coefficients, nonzero monopole and collapsed depth are reported by
    the device status word (physics/shallow_water.py:494-539)."""
    L = 15
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=L)
    s0, depth = W.perturbed_williamson2(L, seed=1)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    model.validate_state(ShallowWaterState(T(s0)))
    bad = s0.copy()
    bad[1, 3, 2] = np.nan
    with pytest.raises(ShallowWaterStateError, match="NaN"):
        model.validate_state(ShallowWaterState(T(bad)))
    bad = s0.copy()
    bad[2, 0, 0] = 1.0
    with pytest.raises(ShallowWaterStateError, match="monopole"):
        model.validate_state(ShallowWaterState(T(bad)))
    bad = s0.copy()
    bad[2, 1, 0] = -3.0 * model.phi0
    with pytest.raises(ShallowWaterStateError, match="thickness"):
        model.validate_state(ShallowWaterState(T(bad)))
    with pytest.raises(ShallowWaterStateError, match="thickness"):
        model.rk4(T(bad), 300.0, 1)


# ------------------------------------------------------------- geodesic
def test_geodesic_golden(golden):
    g = golden("geodesic_res3_L10")
    planet = ae.make_planet("geodesic", resolution=3, l_max=10, product_quadrature="coarse")
    sh = planet.sh
    np.testing.assert_allclose(N(sh.latitudes), g["lat"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(N(sh.weights), g["weights"], rtol=1e-12)
    assert rel_l2(N(sh.inv_transform(T(g["coeffs"]))), g["synth"]) < TOL
    assert rel_l2(N(sh.transform(T(g["field"]))), g["analysis"]) < TOL
    model = BarotropicVorticity(planet)
    assert rel_l2(N(model.tendency(BarotropicState(T(g["zeta"])))), g["bve_tendency"]) < TOL


def test_geodesic_fine_cogrid_golden(golden):
    """Geodesic BVE and SWE with products on the resolution r+1 co-grid
    (the reference's 'fine' geodesic product space): tendencies, RK4 steps,
    co-grid points/weights and geopotential extrema over both samplings."""
    g = golden("geodesic_fine_res3_L10")
    planet = ae.make_planet("geodesic", resolution=int(g["res"]), l_max=int(g["lmax"]),
                            product_quadrature="fine")
    ps = planet.so.backend.product_space("fine")
    assert ps.sh.latitudes.numel() == g["fine_lat"].size
    np.testing.assert_allclose(N(ps.sh.latitudes), g["fine_lat"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(N(ps.sh.longitudes), g["fine_lon"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(N(ps.sh.weights), g["fine_weights"], rtol=1e-12)
    assert planet.grid.cfl_length_scale == pytest.approx(float(g["cfl_length_scale"]), rel=1e-14)
    dt = float(g["dt"])
    bve = BarotropicVorticity(planet, viscosity=1e5)
    z = T(g["zeta"])
    assert rel_l2(tri(N(bve.tendency(BarotropicState(z)))), tri(g["bve_tendency"])) < TOL
    assert rel_l2(tri(N(bve.rk4(z, dt, 1))), tri(g["bve_rk4"])) < TOL
    swe = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    s0 = T(g["state"])
    assert rel_l2(tri(N(swe.tendency(s0))), tri(g["swe_tendency"])) < TOL
    assert rel_l2(tri(N(swe.rk4(s0, dt, 1))), tri(g["swe_rk4"])) < TOL
    np.testing.assert_allclose(swe.total_geopotential_extrema(ShallowWaterState(s0)), g["phi_extrema"],
                               rtol=1e-13)


def test_point_set_batch_matches_oracle():
    rng = np.random.default_rng(8)
    lat = np.arcsin(rng.uniform(-1, 1, 3000))
    lon = rng.uniform(-np.pi, np.pi, 3000)
    w = rng.uniform(0.5, 1.5, 3000)
    L = 20
    p = Plan.points(lat, lon, w, L)
    osh = oracle.PointSetSH(lat, lon, L, weights=w)
    a = np.stack([W.random_spectrum(rng, L, -1.5, 1.0, zero_monopole=False) for _ in range(5)])
    f = rng.standard_normal((5, 3000))
    g = N(synthesize(p.id, T(a)))
    c = N(analyze(p.id, T(f)))
    for b in range(5):
        assert rel_l2(g[b], osh.inv_transform(a[b])) < TOL
        assert rel_l2(tri(c[b]), osh.transform(f[b])) < TOL
