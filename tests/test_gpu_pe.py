"""GPU primitive-equation tendency against the reference's own output and
the oracle restatement.

Golden cases (``tests/golden/pe_*.npz``, made by ``make_golden.py pe`` from
src/planetary_sandbox/physics/primitive_equations.py): a uniform 5-level
sigma grid on a Gauss planet with a distinct 3/2-rule product grid, a
non-uniform 4-level grid with a band-limited surface geopotential, and a
geodesic planet.  Tolerance: 1e-12 relative L2 per prognostic block (the
FP64 drop-in bar).  Exact properties of the reference's own battery
(tests/test_pe_tendency.py): an isothermal resting atmosphere has a zero
tendency, and a barotropic state (no divergence, isothermal, uniform
surface pressure) gives each level the barotropic-vorticity tendency.
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import pe as ope
from helpers import rel_l2, tri

import aeolus_gb300 as ae
from aeolus_gb300.barotropic import BarotropicState, BarotropicVorticity
from aeolus_gb300.primitive_equations import (PrimitiveEquationsModel, PrimitiveEquationsState,
                                              PrimitiveEquationsStateError, SigmaGrid,
                                              isothermal_rest_state)

pytestmark = pytest.mark.gpu
TOL = 1e-12
CASES = {"pe_gauss16x32_L15_fine23x46_K5": ("latlon", dict(nlat=16, nlon=32)),
         "pe_gauss24x48_L15_K4_nonuniform_phis": ("latlon", dict(nlat=24, nlon=48)),
         "pe_geodesic_res3_L10_K3": ("geodesic", dict(resolution=3, product_quadrature="coarse"))}


def T(x):
    return torch.as_tensor(np.asarray(x), device="cuda")


def N(x):
    return x.detach().cpu().numpy()


def _blocks(x, K):
    return [x[..., 0:K, :, :], x[..., K:2 * K, :, :], x[..., 2 * K:3 * K, :, :], x[..., 3 * K, :, :]]


def _model(g, kind, kw):
    planet = ae.make_planet(kind, l_max=int(g["lmax"]), radius=float(g["radius"]), omega=float(g["omega"]), **kw)
    return PrimitiveEquationsModel(planet, SigmaGrid(tuple(g["interfaces"])), r_dry=float(g["r_dry"]),
                                   cp_dry=float(g["cp_dry"]), surface_geopotential_lm=T(g["phi_s"]))


@pytest.mark.parametrize("name", sorted(CASES))
def test_pe_tendency_matches_reference(golden, name):
    g = golden(name)
    m = _model(g, *CASES[name])
    K = m.nlev
    out = N(m.tendency(T(g["state"])))
    for a, b in zip(_blocks(out, K), _blocks(g["tendency"], K)):
        assert rel_l2(tri(a), tri(b)) < TOL


def test_pe_batch_equals_single_calls(golden):
    g = golden("pe_gauss16x32_L15_fine23x46_K5")
    m = _model(g, *CASES["pe_gauss16x32_L15_fine23x46_K5"])
    s = T(g["state"])
    rng = np.random.default_rng(3)
    s2 = s.clone()
    s2[: m.nlev] *= 1.7
    s2[m.nlev:2 * m.nlev] += T(1e-7 * rng.standard_normal(s2[m.nlev:2 * m.nlev].shape))
    batch = m.tendency(torch.stack([s, s2, s]))
    assert torch.equal(batch[0], m.tendency(s)) and torch.equal(batch[1], m.tendency(s2))
    assert torch.equal(batch[0], batch[2])


def test_pe_larger_grid_matches_oracle():
    """Gauss 64x128, l_max 42, 8 non-uniform levels, against the oracle."""
    L, nlat, nlon = 42, 64, 128
    sig = [0.0, 0.05, 0.12, 0.22, 0.35, 0.5, 0.67, 0.84, 1.0]
    R, om = 6.371e6, 7.292e-5
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L, radius=R, omega=om)
    m = PrimitiveEquationsModel(planet, SigmaGrid(tuple(sig)))
    rng = np.random.default_rng(5)
    K, n = 8, L + 1
    s = np.zeros((3 * K + 1, n, n), complex)
    cut = (2 * L) // 3
    for i in range(3 * K + 1):
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        a[:, 0] = a[:, 0].real
        a *= np.tril(np.ones((n, n)))
        a[cut + 1:] = 0
        s[i] = a * (2e-6 if i < 2 * K else (0.5 if i < 3 * K else 1e-3))
    s[2 * K:3 * K, 0, 0] += 250.0 * np.sqrt(4 * np.pi)
    s[3 * K, 0, 0] = np.log(1e5) * np.sqrt(4 * np.pi)
    s[:2 * K, 0, 0] = 0
    nf, mf = oracle.fine_dims(nlat, nlon, L)
    ops = oracle.Operators(oracle.GaussSH(nlat, nlon, L), R, sh_p=oracle.GaussSH(nf, mf, L))
    ref = ope.PE(ops, ope.Sigma(sig), om, oracle.GaussSH(nf, mf, L + 1)).tendency(s)
    out = N(m.tendency(T(s)))
    for a, b in zip(_blocks(out, K), _blocks(ref, K)):
        assert rel_l2(tri(a), tri(b)) < TOL


def test_isothermal_rest_is_exactly_steady():
    planet = ae.make_planet("latlon", nlat=24, nlon=48, l_max=15)
    m = PrimitiveEquationsModel(planet, SigmaGrid.uniform(6))
    st = isothermal_rest_state(15, 6, temperature=260.0, surface_pressure=101325.0)
    assert bool((m.tendency(st.coeffs) == 0).all())


def test_barotropic_state_gives_bve_tendency_per_level():
    L = 15
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=L)
    K = 4
    m = PrimitiveEquationsModel(planet, SigmaGrid.uniform(K))
    st = isothermal_rest_state(L, K, temperature=250.0, surface_pressure=1e5)
    from aeolus_gb300 import workloads as W
    for k in range(K):
        st.coeffs[k] = T(W.bve_vorticity(L, 100 + k))
    out = m.tendency(st.coeffs)
    bve = BarotropicVorticity(planet)
    for k in range(K):
        ref = bve.tendency(BarotropicState(st.coeffs[k]))
        assert rel_l2(tri(N(out[k])), tri(N(ref))) < TOL


def test_pe_rejects_bad_inputs():
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=10)
    m = PrimitiveEquationsModel(planet, SigmaGrid.uniform(3))
    with pytest.raises(PrimitiveEquationsStateError):
        m.tendency(torch.zeros((9, 11, 11), dtype=torch.complex128, device="cuda"))
    with pytest.raises(ValueError):
        m.tendency(torch.zeros((10, 11, 11), dtype=torch.complex128))
    bad = torch.zeros((11, 11), dtype=torch.complex128)
    bad[10, 0] = 1.0
    with pytest.raises(ValueError, match="above the dealiased"):
        PrimitiveEquationsModel(planet, SigmaGrid.uniform(3), surface_geopotential_lm=bad)
    assert m.tendency(torch.zeros((0, 10, 11, 11), dtype=torch.complex128, device="cuda")).shape == (0, 10, 11, 11)


def test_pe_characteristic_speed_and_extrema_match_oracle(golden):
    """max|V| + sqrt(gamma R_d T_max) and the temperature extrema over the
    state and product samplings (primitive_equations.py:764-797)."""
    g = golden("pe_gauss16x32_L15_fine23x46_K5")
    m = _model(g, *CASES["pe_gauss16x32_L15_fine23x46_K5"])
    st = PrimitiveEquationsState(T(g["state"]))
    K, L, R = m.nlev, m.l_max, float(g["radius"])
    sh = oracle.GaussSH(16, 32, L)
    nf, mf = oracle.fine_dims(16, 32, L)
    shp = oracle.GaussSH(nf, mf, L)
    s = g["state"]
    tg = [x.inv_transform(s[2 * K + k]) for x in (sh, shp) for k in range(K)]
    lo, hi = min(t.min() for t in tg), max(t.max() for t in tg)
    assert m.temperature_extrema(st) == pytest.approx((lo, hi), rel=1e-13)
    ops = oracle.Operators(sh, R)
    inv = lambda c: ops.inv_laplacian_zero(c)  # noqa: E731
    cosl = np.maximum(np.cos(sh.latitudes), 1e-8)
    wmax = 0.0
    for k in range(K):
        psi, chi = inv(s[k]), inv(s[K + k])
        lam = lambda c: sh.inv_transform(ops.d_lambda_coeffs(c))  # noqa: E731
        snt = lambda c: sh.inv_transform(ops.sin_theta_d_theta_coeffs(c)) / R  # noqa: E731
        u = (snt(psi) + lam(chi)) / cosl
        v = (lam(psi) - snt(chi)) / cosl
        wmax = max(wmax, float(np.sqrt(u * u + v * v).max()))
    ref = wmax + np.sqrt(m.gamma * m.r_dry * hi)
    assert m.max_characteristic_speed(st) == pytest.approx(ref, rel=1e-12)


def test_pe_validate_state_faults_injected_on_host(golden):
    g = golden("pe_gauss16x32_L15_fine23x46_K5")
    m = _model(g, *CASES["pe_gauss16x32_L15_fine23x46_K5"])
    K = m.nlev
    good = T(g["state"])
    m.validate_state(PrimitiveEquationsState(good))
    cases = []
    x = good.clone(); x[3, 4, 2] = complex(float("nan"), 0.0); cases.append((x, "NaN/Inf"))
    x = good.clone(); x[K + 1, 0, 0] = 1e-3; cases.append((x, "delta monopole is nonzero at level 2"))
    x = good.clone(); x[2 * K + 2, 0, 0] = -10.0; cases.append((x, "temperature is not strictly positive"))
    x = good.clone(); x[3 * K, 0, 0] = 3000.0; cases.append((x, "overflowed"))
    for bad, msg in cases:
        with pytest.raises(PrimitiveEquationsStateError, match=msg):
            m.validate_state(PrimitiveEquationsState(bad), context="in the test")
    with pytest.raises(PrimitiveEquationsStateError, match="does not match"):
        m.validate_state(PrimitiveEquationsState(good[:-3]))


def test_pe_rk4_steps_match_oracle(golden):
    """Two RK4 steps through the generic engine (run/engine.py:406-431) with
    validate_state as the stage validator, against the oracle."""
    from aeolus_gb300.engine import rk4_step_array
    name = "pe_gauss16x32_L15_fine23x46_K5"
    g = golden(name)
    m = _model(g, *CASES[name])
    stages = []

    def validator(y):
        stages.append(1)
        m.validate_state(PrimitiveEquationsState(y), context="in an RK4 stage")

    y = T(g["state"])
    for _ in range(2):
        y = rk4_step_array(m.tendency, y, 0.0, 300.0, stage_validator=validator)
    assert len(stages) == 6
    L, R = int(g["lmax"]), float(g["radius"])
    nf, mf = oracle.fine_dims(16, 32, L)
    ops = oracle.Operators(oracle.GaussSH(16, 32, L), R, sh_p=oracle.GaussSH(nf, mf, L))
    ref_m = ope.PE(ops, ope.Sigma(g["interfaces"]), float(g["omega"]), oracle.GaussSH(nf, mf, L + 1),
                   phi_s_lm=g["phi_s"], r_dry=float(g["r_dry"]), cp_dry=float(g["cp_dry"]))
    from oracle import models as om
    r = g["state"]
    for _ in range(2):
        r = om.rk4_step_array(ref_m.tendency, r, 300.0)
    for a, b in zip(_blocks(N(y), m.nlev), _blocks(r, m.nlev)):
        assert rel_l2(tri(a), tri(b)) < TOL


def test_pe_fused_rk4_is_bitwise_the_generic_engine(golden):
    """model.rk4 (stage combinations fused on the device, aeolus_rk4_stage)
    gives bit for bit the generic engine's rk4_step_array steps (the
    reference's order of operations), with the same stage validations."""
    from aeolus_gb300.engine import rk4_step_array
    name = "pe_gauss16x32_L15_fine23x46_K5"
    g = golden(name)
    m = _model(g, *CASES[name])
    calls = {"a": 0, "b": 0}

    def va(y):
        calls["a"] += 1
        m.validate_state(PrimitiveEquationsState(y), context="in an RK4 stage")

    def vb(y):
        calls["b"] += 1
        m.validate_state(PrimitiveEquationsState(y), context="in an RK4 stage")

    y = T(g["state"])
    ya = y
    for _ in range(3):
        ya = rk4_step_array(m.tendency, ya, 0.0, 300.0, stage_validator=va)
    yb = m.rk4(y, 300.0, 3, stage_validator=vb)
    assert calls["a"] == calls["b"] == 9
    assert torch.equal(ya, yb)


def test_pe_split_precision_matches_fp64():
    """The Legendre contractions on the bf16-digit tensor-core path, the
    degree-(L+1) weak-form vector analysis included (its plan follows the
    product plan's mode): every prognostic within 1e-10 of the FP64 tendency
    at 192x384 / l_max 127, 6 levels."""
    from aeolus_gb300 import _lib
    L, K = 127, 6
    planet = ae.make_planet("latlon", nlat=192, nlon=384, l_max=L)
    m = PrimitiveEquationsModel(planet, SigmaGrid.uniform(K))
    rng = np.random.default_rng(21)
    n, cut = L + 1, (2 * L) // 3
    st = isothermal_rest_state(L, K, temperature=255.0, surface_pressure=1e5).coeffs
    for i in range(3 * K + 1):
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        a[:, 0] = a[:, 0].real
        a *= np.tril(np.ones((n, n)))
        a[cut + 1:] = 0
        if i < 2 * K or i == 3 * K:
            a[0, 0] = 0
        st[i] += T(a * (2e-6 if i < 2 * K else (0.5 if i < 3 * K else 1e-3)))
    t64 = N(m.tendency(st))
    m._plan.set_precision(_lib.PREC_SPLIT_BF16)
    tsp = N(m.tendency(st))
    m._plan.set_precision(_lib.PREC_FP64)
    for a, b in zip(_blocks(tsp, K), _blocks(t64, K)):
        assert rel_l2(a, b) < 1e-10
