"""Split-precision (bf16-digit tcgen05) contraction against the FP64 path.

Tolerances (relative L2 against the FP64 path): 1e-12 for single
transforms (measured ~1e-13); 1e-10 per field for SWE tendencies and RK4
states -- the divergence tendency is a near-cancellation of curl and
Laplacian terms (geostrophic balance), which amplifies the ~1e-13 transform
error by ~100x; 1e-10 is the stated accuracy target of the split form.
"""
import numpy as np
import pytest
import torch

import aeolus_gb300 as ae
from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.ops import Plan, analyze, synthesize
from aeolus_gb300.shallow_water import ShallowWaterModel
from aeolus_gb300.barotropic import BarotropicVorticity, BarotropicState
from helpers import rel_l2

pytestmark = pytest.mark.gpu
DEV = "cuda"


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


def device_error(plan):
    import ctypes
    f = ctypes.c_int()
    _lib.check(_lib.load().aeolus_plan_device_error(plan.handle, ctypes.byref(f)))
    return f.value


@pytest.mark.parametrize("nlat,nlon,L", [(32, 64, 21), (17, 40, 12), (128, 256, 85), (160, 320, 106),
                                         (192, 384, 127), (192, 384, 128), (160, 320, 140)])
def test_split_transforms_match_fp64(nlat, nlon, L):
    """Transforms within 1e-12; l_max 128 (the degree-(L+1) extended plan of
    l_max 127) and 140 give the low orders a second 128-degree analysis tile."""
    rng = np.random.default_rng(L)
    p64 = Plan.gauss(nlat, nlon, L)
    ps = Plan.gauss(nlat, nlon, L)
    ps.set_precision(_lib.PREC_SPLIT_BF16)
    a = np.stack([W.random_spectrum(rng, L, -1.5, 1.0, zero_monopole=False) for _ in range(5)])
    f = rng.standard_normal((5, nlat * nlon))
    g64, gs = N(synthesize(p64.id, T(a))), N(synthesize(ps.id, T(a)))
    c64, cs = N(analyze(p64.id, T(f))), N(analyze(ps.id, T(f)))
    assert device_error(ps) == 0
    for b in range(5):
        assert rel_l2(gs[b], g64[b]) < 1e-12, rel_l2(gs[b], g64[b])
        assert rel_l2(cs[b], c64[b]) < 1e-12, rel_l2(cs[b], c64[b])


def _swe(nlat, nlon, L, precision, members=4, seed=3):
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
    if precision == "split":
        planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    s, depth = W.member_states(L, members, seed=seed)
    return planet, ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth), s


@pytest.mark.parametrize("nlat,nlon,L", [(32, 64, 21), (128, 256, 85), (192, 384, 127), (24, 47, 15),
                                         (80, 160, 52)])
def test_split_swe_tendency_and_steps(nlat, nlon, L):
    """Radix sequences: 64 x 2 (runtime FFT), 128 = (2,8,8) and 192 = (3,8,8)
    (kernels compiled for the sequence), 80 = (5,2,8) (runtime), and an odd
    longitude count (47: direct double-float DFT rows)."""
    _, m64, s = _swe(nlat, nlon, L, "fp64")
    planet, ms, _ = _swe(nlat, nlon, L, "split")
    t64, ts = N(m64.tendency(T(s))), N(ms.tendency(T(s)))
    for b in range(s.shape[0]):
        for f in range(3):
            assert rel_l2(ts[b, f], t64[b, f]) < 1e-10, (b, f, rel_l2(ts[b, f], t64[b, f]))
    y64 = N(m64.rk4(T(s), 240.0, 10))
    ys = N(ms.rk4(T(s), 240.0, 10))
    for b in range(s.shape[0]):
        for f in range(3):
            assert rel_l2(ys[b, f], y64[b, f]) < 1e-10, (b, f, rel_l2(ys[b, f], y64[b, f]))
    assert device_error(planet.so._product_space.sh.plan) == 0


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_rk4_host_streams_equal_device_rk4(precision):
    """ShallowWaterModel.rk4_host (member groups copied in, stepped and copied
    back on streams of their own) gives the device rk4's result bit for bit,
    for any number of groups."""
    _, m, s = _swe(32, 64, 21, precision, members=5, seed=9)
    ref = m.rk4(T(s), 300.0, 2).cpu()
    host = torch.as_tensor(s).pin_memory()
    for chunks in (1, 2, 3):
        out = m.rk4_host(host, 300.0, 2, chunks=chunks)
        torch.cuda.synchronize()
        assert torch.equal(out, ref), chunks


def test_split_bve_matches_fp64():
    L = 63
    p64 = ae.make_planet("latlon", nlat=96, nlon=192, l_max=L)
    ps = ae.make_planet("latlon", nlat=96, nlon=192, l_max=L)
    ps.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    z = np.stack([W.bve_vorticity(L, s) for s in range(6)])
    m64, ms = BarotropicVorticity(p64, viscosity=1e5), BarotropicVorticity(ps, viscosity=1e5)
    t64 = N(m64.tendency(BarotropicState(T(z))))
    ts = N(ms.tendency(BarotropicState(T(z))))
    assert rel_l2(ts, t64) < 1e-12
    assert rel_l2(N(ms.rk4(T(z), 900.0, 5)), N(m64.rk4(T(z), 900.0, 5))) < 1e-11


def test_bounded_wait_gives_up_and_reports():
    """The tensor-core kernels' mbarrier waits are bounded in wall time: a
    wait on a phase that nothing completes gives up after its limit (20 ms
    here), reports it, and leaves the context usable."""
    import ctypes
    flag, ns = ctypes.c_int(-1), ctypes.c_ulonglong(0)
    _lib.check(_lib.load().aeolus_selftest_wait_timeout(20_000_000, ctypes.byref(flag), ctypes.byref(ns)))
    assert flag.value == 1
    assert 20_000_000 <= ns.value < 1_000_000_000
    assert float(torch.ones(4, device=DEV).sum()) == 4.0


def _hi24(x):
    """x truncated to 24 significant bits (the low 29 mantissa bits cleared)."""
    b = np.asarray(x, dtype=np.float64).view(np.uint64) & ~np.uint64((1 << 29) - 1)
    return b.view(np.float64)


def test_double_float_conversions_on_device():
    """The FP64 <-> double-float conversions of the split derive, PE derive
    and column kernels (integer operations on the bits): hi = x truncated
    to 24 bits, lo = the rest rounded to a float, |x - hi - lo| <= 2^-48 |x|,
    and the way back rounds hi + lo once; |x| below 2^-126 gives 0, 2^128
    and above infinity."""
    rng = np.random.default_rng(7)
    mag = 10.0 ** rng.uniform(-25, 30, 20000)  # lo stays a normal float or an exact subnormal
    edge = [1.0, -1.0, 2.0 ** -126, 2.0 ** 127, np.nextafter(2.0 ** 128, 0), 3.0, np.pi,
            np.nextafter(1.0, 2.0), np.nextafter(2.0, 0.0), 1.0 + 2.0 ** -24 - 2.0 ** -52, -np.e * 1e-20]
    x = np.concatenate([mag * rng.choice([-1.0, 1.0], mag.size), edge])
    special = np.array([0.0, -0.0, 2.0 ** -127, -1e-300, 2.0 ** 128, -1e300])
    allx = np.concatenate([x, special])
    d_x = T(allx)
    d_out = torch.empty(3 * allx.size, dtype=torch.float64, device=DEV)
    _lib.check(_lib.load().aeolus_selftest_df_convert(d_x.data_ptr(), allx.size, d_out.data_ptr(),
                                                      torch.cuda.current_stream().cuda_stream))
    out = N(d_out).reshape(-1, 3)
    hi, lo, back = out[: x.size, 0], out[: x.size, 1], out[: x.size, 2]
    np.testing.assert_array_equal(hi, _hi24(x))
    np.testing.assert_array_equal(lo, (x - _hi24(x)).astype(np.float32).astype(np.float64))
    np.testing.assert_array_equal(back, hi + lo)
    assert np.all(np.abs(x - (hi + lo)) <= 2.0 ** -48 * np.abs(x))
    sp = out[x.size:]
    np.testing.assert_array_equal(sp[:4], np.zeros((4, 3)))
    assert sp[4, 0] == np.inf and sp[4, 1] == 0.0 and sp[4, 2] == np.inf
    assert sp[5, 0] == -np.inf and sp[5, 1] == 0.0 and sp[5, 2] == -np.inf


def test_split_rejects_unsupported_shapes():
    p = Plan.gauss(256, 512, 170)
    with pytest.raises(ValueError, match="l_max"):
        p.set_precision(_lib.PREC_SPLIT_BF16)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_swe_autotune_is_bitwise_neutral(precision):
    """Launch shapes picked by the autotuner change no result bit."""
    L = 85
    planet = ae.make_planet("latlon", nlat=128, nlon=256, l_max=L)
    if precision == "split":
        planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    s, depth = W.member_states(L, 5, seed=21)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    y0 = torch.as_tensor(s, device="cuda")
    before = model.rk4(y0, 300.0, 2, check=False)
    out = model.autotune(y0, 300.0, reps=1)
    assert len(out["chosen"]) == 5 and out["ms_per_step"] > 0
    after = model.rk4(y0, 300.0, 2, check=False)
    assert torch.equal(before, after)


@pytest.mark.parametrize("nlat,nlon,L", [(96, 192, 63), (16, 1024, 15), (24, 47, 15), (192, 384, 127)])
@pytest.mark.parametrize("scale", [1.0, 1e-20, 1e20])
def test_split_worst_case_growth_matches_fp64(nlat, nlon, L, scale):
    """Inputs that drive the longitude transforms to their largest growth: a
    spectral delta (every order adds in phase at one grid point, the largest
    value an inverse FFT can reach from its spectra) and grid rows that are
    constant along longitude (the whole row sums into order 0), at extreme
    magnitudes.  The fixed-point row stage picks its block exponents so that
    no butterfly overflows; the results must stay within 1e-12 of FP64.
    Includes a 512-point FFT and a 47-point direct DFT."""
    p64 = Plan.gauss(nlat, nlon, L)
    ps = Plan.gauss(nlat, nlon, L)
    ps.set_precision(_lib.PREC_SPLIT_BF16)
    delta = np.zeros((2, nlat * nlon))
    delta[0, (nlat // 3) * nlon] = scale
    delta[1, (nlat // 2) * nlon + nlon // 5] = -scale
    a = analyze(p64.id, T(delta))
    g64, gs = N(synthesize(p64.id, a)), N(synthesize(ps.id, a))
    rows = np.zeros((2, nlat, nlon))
    rows[0, nlat // 4, :] = scale
    rows[1, :, :] = scale * np.cos(np.linspace(0.0, 3.0, nlat))[:, None]
    rows = rows.reshape(2, -1)
    c64, cs = N(analyze(p64.id, T(rows))), N(analyze(ps.id, T(rows)))
    assert device_error(ps) == 0
    for b in range(2):
        assert rel_l2(gs[b], g64[b]) < 1e-12, (b, rel_l2(gs[b], g64[b]))
        assert rel_l2(cs[b], c64[b]) < 1e-12, (b, rel_l2(cs[b], c64[b]))


def test_c2_williamson2_100_steps_split_vs_fp64():
    """The shallow-water plain-vs-split workload: Gauss 128x256, l_max 85,
    Williamson-2 plus the seeded 1 % perturbation, dt = 300 s, 100 RK4 steps
    on both paths; every field within 1e-10 relative L2 of the FP64 path."""
    L, nlat, nlon = 85, 128, 256
    s0, depth = W.perturbed_williamson2(L, seed=2)
    out = {}
    for prec in ("fp64", "split"):
        planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L)
        if prec == "split":
            planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
        m = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
        out[prec] = N(m.rk4(T(s0), 300.0, 100))
    for f in range(3):
        err = rel_l2(out["split"][f], out["fp64"][f])
        assert err < 1e-10, (f, err)
    assert np.isfinite(out["fp64"]).all()
