"""Pin the CPU oracle against golden vectors made by the reference itself.

Fixtures: tests/golden/*.npz from tests/golden/make_golden.py (reference code
run on the CPU).  Tolerances: 1e-12 relative L2 for float64 transforms and
tendencies (the bar the FP64 GPU path must meet as well).
"""
import numpy as np
import pytest

import oracle
from oracle import models, diagnostics
from helpers import rel_l2

TOL = 1e-12


def gauss_ops(nlat, nlon, lmax, R):
    sh = oracle.GaussSH(nlat, nlon, lmax)
    nf, mf = oracle.fine_dims(nlat, nlon, lmax)
    sh_p = sh if (nf, mf) == (nlat, nlon) else oracle.GaussSH(nf, mf, lmax)
    return oracle.Operators(sh, R, sh_p=sh_p)


@pytest.mark.parametrize("name", ["bve_gauss32x64_L21", "bve_gauss16x32_L15_fine23x46"])
def test_bve_golden(golden, name):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    ops = gauss_ops(nlat, nlon, L, float(g["radius"]))
    assert tuple(g["product_grid"]) == oracle.fine_dims(nlat, nlon, L)
    np.testing.assert_allclose(ops.sh.lat, g["lat"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(ops.sh.weights, g["weights"], rtol=1e-14)
    zeta = g["zeta"]
    assert rel_l2(ops.sh.inv_transform(zeta), g["grid"]) < TOL
    assert rel_l2(ops.sh.transform(g["grid"]), g["roundtrip"]) < TOL
    om, nu, dt = float(g["omega"]), float(g["nu"]), float(g["dt"])
    assert rel_l2(models.bve_tendency(ops, zeta, om, nu), g["tendency"]) < TOL
    step = models.bve_rk4_step(ops, zeta, dt, om, nu)
    assert rel_l2(step, g["rk4"]) < TOL
    keys = list(g["spec_keys"])
    d0 = diagnostics.spectral_diagnostics(zeta, ops.R, om)
    d1 = diagnostics.spectral_diagnostics(step, ops.R, om)
    for k, v0, v1 in zip(keys, g["spec0"], g["spec1"]):
        assert d0[k] == pytest.approx(v0, rel=1e-12, abs=1e-300)
        assert d1[k] == pytest.approx(v1, rel=1e-10, abs=1e-300)
    dg = diagnostics.grid_diagnostics(zeta, ops.sh, ops.R, om)
    for k, v in zip(list(g["grid_keys"]), g["grid0"]):
        assert dg[k] == pytest.approx(v, rel=1e-11, abs=1e-3)


@pytest.mark.parametrize("name", ["swe_gauss16x32_L15_fine23x46", "swe_gauss32x64_L21",
                                  "swe_gauss128x256_L85"])
def test_swe_golden(golden, name):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    ops = gauss_ops(nlat, nlon, L, float(g["radius"]))
    m = models.SWE(ops, float(g["omega"]), float(g["gravity"]), float(g["mean_depth"]))
    s = g["state"]
    assert rel_l2(m.tendency(s), g["tendency"]) < TOL
    u, v = m.wind_on_state_grid(s)
    assert rel_l2(u, g["u"]) < TOL and rel_l2(v, g["v"]) < TOL
    np.testing.assert_allclose(m.total_geopotential_extrema(s), g["phi_extrema"], rtol=1e-13)
    if L <= 21:
        y = s
        for _ in range(int(g["steps"])):
            y = models.rk4_step_array(m.tendency, y, float(g["dt"]))
        assert rel_l2(y, g["rk4"]) < TOL


def test_geodesic_golden(golden):
    g = golden("geodesic_res3_L10")
    lat, lon, w = oracle.geodesic.geodesic_point_set(int(g["res"]), float(g["radius"]))
    np.testing.assert_allclose(lat, g["lat"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(lon, g["lon"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(w, g["weights"], rtol=1e-12)
    sh = oracle.PointSetSH(lat, lon, int(g["lmax"]), weights=w)
    assert rel_l2(sh.inv_transform(g["coeffs"]), g["synth"]) < TOL
    assert rel_l2(sh.transform(g["field"]), g["analysis"]) < TOL
    ops = oracle.Operators(sh, float(g["radius"]))
    t = models.bve_tendency(ops, g["zeta"], float(g["omega"]))
    assert rel_l2(t, g["bve_tendency"]) < TOL


def test_geodesic_fine_cogrid_golden(golden):
    """Geodesic planet whose products are formed on the resolution r+1
    co-grid (spherical_backend.py:159-168): BVE and SWE tendencies and RK4
    steps of the reference, restated."""
    g = golden("geodesic_fine_res3_L10")
    res, L, R = int(g["res"]), int(g["lmax"]), float(g["radius"])
    lat, lon, w = oracle.geodesic.geodesic_point_set(res, R)
    flat, flon, fw = oracle.geodesic.geodesic_point_set(res + 1, R)
    np.testing.assert_allclose(flat, g["fine_lat"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(flon, g["fine_lon"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(fw, g["fine_weights"], rtol=1e-12)
    sh = oracle.PointSetSH(lat, lon, L, weights=w)
    ops = oracle.Operators(sh, R, sh_p=oracle.PointSetSH(flat, flon, L, weights=fw))
    om, dt = float(g["omega"]), float(g["dt"])
    assert rel_l2(models.bve_tendency(ops, g["zeta"], om, 1e5), g["bve_tendency"]) < TOL
    assert rel_l2(models.bve_rk4_step(ops, g["zeta"], dt, om, 1e5), g["bve_rk4"]) < TOL
    m = models.SWE(ops, om, float(g["gravity"]), float(g["mean_depth"]))
    assert rel_l2(m.tendency(g["state"]), g["swe_tendency"]) < TOL
    assert rel_l2(models.rk4_step_array(m.tendency, g["state"], dt), g["swe_rk4"]) < TOL


PE_CASES = {"pe_gauss16x32_L15_fine23x46_K5": ("gauss", 16, 32),
            "pe_gauss24x48_L15_K4_nonuniform_phis": ("gauss", 24, 48),
            "pe_geodesic_res3_L10_K3": ("geodesic", 3, None)}


def pe_oracle(g, kind, a, b):
    """Oracle PE model on the planet the golden case was made on."""
    from oracle import pe as ope
    L, R = int(g["lmax"]), float(g["radius"])
    if kind == "gauss":
        nf, mf = oracle.fine_dims(a, b, L)
        ops = gauss_ops(a, b, L, R)
        sh_ext = oracle.GaussSH(nf, mf, L + 1)
    else:
        lat, lon, w = oracle.geodesic.geodesic_point_set(a, R)
        sh = oracle.PointSetSH(lat, lon, L, weights=w)
        ops = oracle.Operators(sh, R)
        sh_ext = oracle.PointSetSH(lat, lon, L + 1, weights=w)
    return ope.PE(ops, ope.Sigma(g["interfaces"]), float(g["omega"]), sh_ext, phi_s_lm=g["phi_s"],
                  r_dry=float(g["r_dry"]), cp_dry=float(g["cp_dry"]))


@pytest.mark.parametrize("name", sorted(PE_CASES))
def test_pe_tendency_golden(golden, name):
    """Dry hydrostatic primitive-equation tendency (primitive_equations.py:
    727-753) against the reference's own output: uniform and non-uniform
    sigma grids, a band-limited surface geopotential, a distinct 3/2-rule
    product grid and a geodesic planet."""
    g = golden(name)
    m = pe_oracle(g, *PE_CASES[name])
    assert rel_l2(m.tendency(g["state"]), g["tendency"]) < TOL


def test_swe_topography_golden(golden):
    """Shallow water over the reference's Gaussian mountain (its terrain
    coefficients taken from the golden file): tendency and RK4 steps, with
    and without hyperdiffusion."""
    g = golden("topo_swe_gauss32x64_L21_mountain")
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    ops = gauss_ops(nlat, nlon, L, float(g["radius"]))
    for key, nu4 in (("plain", 0.0), ("nu4", float(g["nu4"]))):
        m = models.SWE(ops, float(g["omega"]), float(g["gravity"]), float(g["mean_depth"]), nu4=nu4,
                       elevation_lm=g["elevation_lm"])
        assert rel_l2(m.tendency(g["state"]), g[f"tendency_{key}"]) < TOL
        y = g["state"]
        for _ in range(int(g["steps"])):
            y = models.rk4_step_array(m.tendency, y, float(g["dt"]))
        assert rel_l2(y, g[f"rk4_{key}"]) < TOL


def test_factored_equals_dense():
    """GaussSH (Legendre + DFT) equals PointSetSH (reference dense form)."""
    rng = np.random.default_rng(1)
    for nlat, nlon, L in [(16, 32, 15), (23, 46, 15), (24, 48, 10)]:
        gs = oracle.GaussSH(nlat, nlon, L)
        ps = oracle.PointSetSH(gs.latitudes, gs.longitudes, L, weights=gs.weights)
        a = rng.standard_normal((L + 1, L + 1)) + 1j * rng.standard_normal((L + 1, L + 1))
        f = rng.standard_normal(nlat * nlon)
        assert rel_l2(gs.inv_transform(a), ps.inv_transform(a)) < 1e-13
        assert rel_l2(gs.transform(f), ps.transform(f)) < 1e-13


def test_basis_matches_scipy():
    """Normalised recurrence == scipy.special.sph_harm_y, including l_max=127."""
    sp = pytest.importorskip("scipy.special")
    if not hasattr(sp, "sph_harm_y"):
        pytest.skip("scipy too old")
    rng = np.random.default_rng(2)
    lat = rng.uniform(-1.55, 1.55, 7)
    lon = rng.uniform(0, 2 * np.pi, 7)
    L = 127
    Y = oracle.dense_basis(lat, lon, L)
    for l in (0, 1, 40, 85, 100, 127):
        for m in sorted({0, min(1, l), l // 2, l}):
            ref = sp.sph_harm_y(l, m, np.pi / 2 - lat, lon)
            k = l * (l + 1) // 2 + m
            assert np.allclose(Y[:, k], ref, rtol=1e-10, atol=1e-14), (l, m)


@pytest.mark.parametrize("name", ["vector_gauss16x32_L15_fine23x46", "vector_geodesic_res3_L10"])
def test_vector_curl_div_golden(golden, name):
    """Weak-form curl/div with one-degree-extended analyses
    (spectral_operators.py:399-492) against the reference's own output."""
    g = golden(name)
    L, R = int(g["lmax"]), float(g["radius"])
    lat, lon, w = g["lat"], g["lon"], g["weights"]
    sh_p = oracle.PointSetSH(lat, lon, L, weights=w)
    sh_ext = oracle.PointSetSH(lat, lon, L + 1, weights=w)
    ops = oracle.Operators(sh_p, R, sh_p=sh_p)
    curl, div = ops.vector_curl_div_spectral(g["f_east"], g["f_north"], sh_ext)
    assert rel_l2(curl, g["curl"]) < TOL
    assert rel_l2(div, g["div"]) < TOL


def test_vector_curl_div_recovers_potentials():
    """On the 3/2-rule Gauss product grid the weak integrands of fields built
    from band-limited potentials are integrated exactly: curl = lap(psi),
    div = lap(chi) to round-off (the property the reference documents at
    spectral_operators.py:433-437)."""
    L, R = 12, 6.371e6
    nf, mf = oracle.fine_dims(L + 1, 2 * L + 2, L)
    sh_p = oracle.GaussSH(nf, mf, L)
    ops = oracle.Operators(oracle.GaussSH(L + 1, 2 * L + 2, L), R, sh_p=sh_p)
    rng = np.random.default_rng(0)
    cut = (2 * L) // 3
    psi = np.zeros((L + 1, L + 1), complex)
    chi = np.zeros_like(psi)
    for a in (psi, chi):
        for l in range(1, cut + 1):
            a[l, 1:l + 1] = rng.standard_normal(l) + 1j * rng.standard_normal(l)
            a[l, 0] = rng.standard_normal()
    snt = lambda c: sh_p.inv_transform(ops.sin_theta_d_theta_coeffs(c)) / R
    lam = lambda c: sh_p.inv_transform(ops.d_lambda_coeffs(c))
    u = (snt(psi) + lam(chi)) / ops.coslat_p   # shallow_water.py:305-319 winds
    v = (lam(psi) - snt(chi)) / ops.coslat_p
    curl, div = ops.vector_curl_div_spectral(u, v, oracle.GaussSH(nf, mf, L + 1))
    assert rel_l2(curl, ops.laplacian_coeffs(psi)) < 1e-13
    assert rel_l2(div, ops.laplacian_coeffs(chi)) < 1e-13
