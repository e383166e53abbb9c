"""Weak-form curl/div of tangent fields with one-degree-extended analyses
(spectral_operators.py:399-492, vector_curl_div_spectral) on the GPU.

Parity: against the reference's own output (golden fixtures made by
tests/golden/make_golden.py) at 1e-12 relative L2; through the Python mirror
(SpectralOperators on a 3/2-rule Gauss product space); and the property the
reference documents -- on the Gauss product grid, fields built from
band-limited potentials give curl = lap(psi), div = lap(chi) to round-off --
at l_max 85 and 127 (tolerance 1e-12).
"""
import numpy as np
import pytest
import torch

import aeolus_gb300 as ae
from aeolus_gb300 import _lib
from aeolus_gb300.ops import Plan, spectral_op, synthesize, vector_curl_div
from helpers import rel_l2, tri

pytestmark = pytest.mark.gpu
DEV = "cuda"


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("name", ["vector_gauss16x32_L15_fine23x46", "vector_geodesic_res3_L10"])
def test_vector_curl_div_matches_reference(golden, name):
    g = golden(name)
    L, R = int(g["lmax"]), float(g["radius"])
    if "gauss" in name:
        plan = Plan.gauss(23, 46, L + 1, R)
        assert plan.n_points == g["lat"].size
    else:
        plan = Plan.points(g["lat"], g["lon"], g["weights"], L + 1, R)
    out = N(vector_curl_div(plan.id, R, T(g["f_east"]), T(g["f_north"]), True))
    assert rel_l2(out[0], g["curl"]) < 1e-12, rel_l2(out[0], g["curl"])
    assert rel_l2(out[1], g["div"]) < 1e-12, rel_l2(out[1], g["div"])


def test_vector_curl_div_through_spectral_operators(golden):
    """The mirror's SpectralOperators.vector_curl_div_spectral on the 'fine'
    product space of a Gauss 16x32 / l_max 15 planet (a 23x46 product grid)."""
    g = golden("vector_gauss16x32_L15_fine23x46")
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=15)
    so = planet.so
    curl, div = so.vector_curl_div_spectral(g["f_east"], g["f_north"])
    assert rel_l2(N(curl), g["curl"]) < 1e-12
    assert rel_l2(N(div), g["div"]) < 1e-12
    # truncate=False keeps the rows above the 2/3 cut
    curl_full, _ = so.vector_curl_div_spectral(g["f_east"], g["f_north"], truncate=False)
    cut = (2 * 15) // 3
    assert float(torch.linalg.vector_norm(curl_full[cut + 1:, :])) > 0.0
    torch.testing.assert_close(curl_full[:cut + 1, :cut + 1], curl[:cut + 1, :cut + 1], rtol=0, atol=0)


@pytest.mark.parametrize("nlat,nlon,L", [(128, 256, 85), (192, 384, 127)])
def test_vector_curl_div_recovers_potentials(nlat, nlon, L):
    R = 6.371e6
    nf, mf = max(3 * L // 2 + 1, nlat), max(3 * L + 1, nlon)  # 3/2-rule product grid, spherical_backend.py:201-203
    pp = Plan.gauss(nf, mf, L, R)          # product grid at the state degree
    pe = Plan.gauss(nf, mf, L + 1, R)      # the same points, one degree more
    rng = np.random.default_rng(L)
    cut = (2 * L) // 3
    pots = np.zeros((2, 3, L + 1, L + 1), complex)  # 3 members of (psi, chi)
    for l in range(1, cut + 1):
        pots[:, :, l, :l + 1] = (rng.standard_normal((2, 3, l + 1)) + 1j * rng.standard_normal((2, 3, l + 1)))
    pots[:, :, :, 0] = pots[:, :, :, 0].real
    psi, chi = T(pots[0]), T(pots[1])
    snt = lambda c: synthesize(pp.id, spectral_op(_lib.SOP_SIN_THETA_D_THETA, R, c)) / R
    lam = lambda c: synthesize(pp.id, spectral_op(_lib.SOP_D_LAMBDA, R, c))
    cos = torch.clamp(torch.cos(T(np.repeat(pp.nodes()[0], mf))), min=1e-8)
    u = (snt(psi) + lam(chi)) / cos          # shallow_water.py:305-319 winds
    v = (lam(psi) - snt(chi)) / cos
    out = vector_curl_div(pe.id, R, u, v, True)
    lap = lambda c: spectral_op(_lib.SOP_LAPLACIAN, R, c)
    assert rel_l2(N(out[0]), N(lap(psi))) < 1e-12, rel_l2(N(out[0]), N(lap(psi)))
    assert rel_l2(N(out[1]), N(lap(chi))) < 1e-12, rel_l2(N(out[1]), N(lap(chi)))


def test_vector_curl_div_rejects_bad_arguments():
    p = Plan.gauss(24, 48, 16)
    x = torch.zeros(p.n_points, dtype=torch.float64, device=DEV)
    with pytest.raises(ValueError):
        vector_curl_div(p.id, 1.0, x, x[:-1], True)
    with pytest.raises(Exception):
        vector_curl_div(p.id, -1.0, x, x, True)


def test_roundtrip_curl_div_matches_reference(golden):
    """The reference's scalar round-trip pathway (spectral_operators.py:336-397)
    on the 23x46 product grid of a Gauss 16x32 / l_max 15 planet."""
    g = golden("misc_gauss16x32_L15")
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=15)
    curl, div = planet.so.vector_curl_div_roundtrip(g["f_east"], g["f_north"])
    assert rel_l2(tri(curl.cpu().numpy()), tri(g["rt_curl"])) < 1e-12
    assert rel_l2(tri(div.cpu().numpy()), tri(g["rt_div"])) < 1e-12


def test_vector_curl_div_split_extended_plan_matches_fp64():
    """The weak-form curl/div on the degree-128 extended plan of the 192x384 /
    l_max 127 grid in split precision (order 0, with 129 degrees, takes a
    second degree tile in the tensor-core analysis) against the FP64 plan, within 1e-12 of
    the FP64 result (truncated and full)."""
    R, L = 6.371e6, 127
    p64 = Plan.gauss(192, 384, L + 1, R)
    ps = Plan.gauss(192, 384, L + 1, R)
    ps.set_precision(_lib.PREC_SPLIT_BF16)
    rng = np.random.default_rng(9)
    fe = T(rng.standard_normal((4, p64.n_points)))
    fn = T(rng.standard_normal((4, p64.n_points)))
    for trunc in (True, False):
        a = N(vector_curl_div(p64.id, R, fe, fn, trunc))
        b = N(vector_curl_div(ps.id, R, fe, fn, trunc))
        for k in range(2):
            assert rel_l2(b[k], a[k]) < 1e-12, (trunc, k, rel_l2(b[k], a[k]))
