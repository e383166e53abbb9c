"""Split-precision (bf16-digit tcgen05) dense basis products of point-set
plans against the FP64 basis products, from small weighted point sets to the
icosahedral level-6 grid at l_max 127 with 64 fields (40,962 points, 16,384
real basis columns).  Tolerance: 1e-12 relative L2 per field, 5e-12 for the
level-6 / l_max 127 products whose sums run over 16,384 and 40,962 terms
(the error is that of the dropped digit levels, ~2^-47 of sum |b||v| per
output; measured 1.6e-12)."""
import math

import numpy as np
import pytest
import torch

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.barotropic import BarotropicState, BarotropicVorticity
from aeolus_gb300.ops import Plan, analyze, synthesize
from helpers import rel_l2

pytestmark = pytest.mark.gpu
DEV = "cuda"


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


def _pair(lat, lon, w, L):
    a = Plan.points(lat, lon, w, L)
    b = Plan.points(lat, lon, w, L)
    b.set_precision(_lib.PREC_SPLIT_BF16)
    return a, b


def _check(p64, psp, L, nf, seed, tol=1e-12):
    rng = np.random.default_rng(seed)
    a = np.stack([W.random_spectrum(rng, L, -1.5, 1.0, zero_monopole=False) for _ in range(nf)])
    g64 = synthesize(p64.id, T(a))
    gsp = synthesize(psp.id, T(a))
    c64 = analyze(p64.id, g64)
    csp = analyze(psp.id, g64)
    errs = []
    for f in range(nf):
        errs.append((rel_l2(N(gsp[f]), N(g64[f])), rel_l2(N(csp[f]), N(c64[f]))))
    worst = max(max(e) for e in errs)
    assert worst < tol, worst
    return worst


def test_random_weighted_point_set():
    rng = np.random.default_rng(3)
    n, L = 900, 12
    lat = np.arcsin(rng.uniform(-1, 1, n))
    lon = rng.uniform(-math.pi, math.pi, n)
    w = rng.uniform(0.5, 1.5, n)
    w *= 4 * math.pi / w.sum()
    p64, psp = _pair(lat, lon, w, L)
    _check(p64, psp, L, 3, 1)


def test_geodesic_bve_tendency_split_matches_fp64():
    L = 21
    models = []
    for prec in ("fp64", "split"):
        planet = ae.make_planet("geodesic", resolution=4, l_max=L)
        if prec == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        models.append(BarotropicVorticity(planet, viscosity=1e5))
    z = T(np.stack([W.bve_vorticity(L, s) for s in range(3)]))
    t64 = models[0].tendency(BarotropicState(z))
    tsp = models[1].tendency(BarotropicState(z))
    assert rel_l2(N(tsp), N(t64)) < 1e-11


def test_geodesic_level6_lmax127_64_fields():
    """Config c3: synthesis and quadrature analysis of 64 fields on the
    level-6 icosahedral grid with Voronoi weights."""
    from aeolus_gb300.geodesic_grid import GeodesicGridGeometry, GeodesicSphericalHarmonics
    sh = GeodesicSphericalHarmonics(GeodesicGridGeometry(6, 6.371e6), 127, weights="voronoi")
    p64 = sh.plan
    assert p64.n_points == 40962
    psp = Plan.points(N(sh.latitudes), N(sh.longitudes), N(sh.weights), 127)
    psp.set_precision(_lib.PREC_SPLIT_BF16)
    _check(p64, psp, 127, 64, 7, tol=5e-12)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_weighted_least_squares_analysis_matches_dense_lstsq(precision):
    """WLS analysis (preconditioned CG on the normal equations with the
    plan's own products) against numpy's weighted least squares on the
    oracle's dense basis; irregular points, so the quadrature analysis alone
    is not the least-squares fit.  Tolerance 1e-9 relative L2."""
    import oracle
    from aeolus_gb300.wls import wls_analysis
    rng = np.random.default_rng(11)
    n, L = 900, 12
    lat = np.arcsin(rng.uniform(-1, 1, n))
    lon = rng.uniform(-math.pi, math.pi, n)
    w = rng.uniform(0.5, 1.5, n)
    w *= 4 * math.pi / w.sum()
    p = Plan.points(lat, lon, w, L)
    if precision == "split":
        p.set_precision(_lib.PREC_SPLIT_BF16)
    f = rng.standard_normal((2, n))
    a, iters, res = wls_analysis(p, T(f), iters=60, rtol=1e-13)
    assert float(res.max()) < 1e-11 and iters < 60
    # real design matrix of the synthesis f = sum Re Y_l0 Re a_l0 + 2 Re(Y_lm a_lm)
    Y = oracle.sht.dense_basis(lat, lon, L)
    cols, idx = [], []
    for l in range(L + 1):
        for m in range(l + 1):
            y = Y[:, l * (l + 1) // 2 + m]
            if m == 0:
                cols.append(y.real)
                idx.append((l, m, 0))
            else:
                cols += [2 * y.real, -2 * y.imag]
                idx += [(l, m, 0), (l, m, 1)]
    D = np.stack(cols, axis=1)
    sw = np.sqrt(w)[:, None]
    ref = np.linalg.lstsq(sw * D, (sw * f.T), rcond=None)[0]
    got = N(a)
    out = np.zeros_like(ref)
    for k, (l, m, c) in enumerate(idx):
        out[k] = got[:, l, m].imag if c else got[:, l, m].real
    assert rel_l2(out, ref) < 1e-9
    # and the quadrature analysis is not the least-squares fit on these points
    q = N(analyze(p.id, T(f)))
    qv = np.array([q[:, l, m].imag if c else q[:, l, m].real for (l, m, c) in idx])
    assert rel_l2(qv, ref) > 1e-3
