"""Shallow water over bottom topography against the reference.

Golden file ``tests/golden/topo_swe_gauss32x64_L21_mountain.npz`` (made by
``make_golden.py topo``): the reference's Gaussian mountain
(physics/topography.py:207-292) on a Gauss 32x64 / l_max 21 planet, the
shallow-water tendency and two RK4 steps over it with and without
hyperdiffusion (shallow_water.py:397-413), and a run capsule of its
run_swe.  FP64 bar 1e-12 relative L2; the split path within 1e-10.
"""
import numpy as np
import pytest
import torch

from helpers import rel_l2, tri

import aeolus_gb300 as ae
from aeolus_gb300 import _lib
from aeolus_gb300 import runner as RN
from aeolus_gb300.shallow_water import ShallowWaterModel, ShallowWaterState
from aeolus_gb300.topography import Topography, TopographyError

pytestmark = pytest.mark.gpu
DEV = "cuda"
TOL = 1e-12


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)


def N(x):
    return x.detach().cpu().numpy()


def _setup(g, precision="fp64"):
    planet = ae.make_planet("latlon", nlat=int(g["nlat"]), nlon=int(g["nlon"]), l_max=int(g["lmax"]), device=DEV)
    if precision == "split":
        planet.so._product_space.sh.plan.set_precision(_lib.PREC_SPLIT_BF16)
    topo = Topography.mountain(planet, height_m=float(g["height_m"]), lat_deg=float(g["lat_deg"]),
                               lon_deg=float(g["lon_deg"]), width_deg=float(g["width_deg"]))
    return planet, topo


def test_mountain_matches_reference(golden):
    g = golden("topo_swe_gauss32x64_L21_mountain")
    planet, topo = _setup(g)
    assert not topo.is_flat and topo.preset == "mountain"
    assert rel_l2(tri(N(topo.elevation_lm)), tri(g["elevation_lm"])) < TOL
    m = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]), topography=topo)
    np.testing.assert_allclose(m.surface_elevation_extrema, g["elevation_extrema"], rtol=1e-9, atol=1e-9)
    with pytest.raises(TopographyError, match="narrow"):
        Topography.mountain(planet, height_m=1000.0, lat_deg=0.0, lon_deg=0.0, width_deg=1.0)
    with pytest.raises(TopographyError):
        Topography.mountain(planet, height_m=-5.0, lat_deg=0.0, lon_deg=0.0, width_deg=20.0)


@pytest.mark.parametrize("key", ["plain", "nu4"])
def test_swe_tendency_and_steps_over_mountain(golden, key):
    g = golden("topo_swe_gauss32x64_L21_mountain")
    nu4 = float(g["nu4"]) if key == "nu4" else 0.0
    for precision, tol in (("fp64", TOL), ("split", 1e-10)):
        planet, topo = _setup(g, precision)
        m = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]),
                              hyperdiffusion_nu4=nu4, topography=topo)
        s = T(g["state"])
        assert rel_l2(tri(N(m.tendency(s))), tri(g[f"tendency_{key}"])) < tol, precision
        y = m.rk4(s, float(g["dt"]), int(g["steps"]))
        assert rel_l2(tri(N(y)), tri(g[f"rk4_{key}"])) < tol, precision


def test_lake_at_rest_is_steady():
    """u = 0 and phi = -phi_s' (flat free surface): zero tendency up to the
    rounding of the two cancelling terms."""
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=21, device=DEV)
    topo = Topography.mountain(planet, height_m=1500.0, lat_deg=-20.0, lon_deg=45.0, width_deg=25.0)
    for nu4 in (0.0, 1e16):
        m = ShallowWaterModel(planet, gravity=9.80616, mean_depth=8000.0, hyperdiffusion_nu4=nu4, topography=topo)
        s = torch.zeros((3, 22, 22), dtype=torch.complex128, device=DEV)
        s[2] = -m.phi_s_anom_lm
        t = m.tendency(s)
        scale = float((m.lap_eigs[:, None] * m.phi_s_lm).abs().max())
        assert float(t.abs().max()) <= 1e-13 * scale
        y = m.rk4(s, 600.0, 3)
        assert float((y - s).abs().max()) <= 1e-12 * float(s.abs().max())


def test_flat_topography_is_the_flat_path():
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=21, device=DEV)
    from aeolus_gb300 import workloads as W
    s0, depth = W.perturbed_williamson2(21, seed=4)
    a = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    b = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth, topography=Topography.flat(21))
    assert b.forcing is None and not b.has_topography
    assert torch.equal(a.rk4(T(s0), 300.0, 2), b.rk4(T(s0), 300.0, 2))


def test_swe_run_over_mountain_matches_reference_runner(golden, tmp_path):
    g = golden("topo_swe_gauss32x64_L21_mountain")
    planet, topo = _setup(g)
    m = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]), topography=topo)
    RN.run_swe(m, ShallowWaterState(T(g["state"])), None, float(g["t_end_days"]), tmp_path,
               snapshot_times=list(g["snapshot_times"]), snapshot_mode="count", plots=())
    times = np.load(tmp_path / "swe_snapshot_times.npy")
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "swe_coeffs.npy")
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= TOL
    import csv
    with open(tmp_path / "diagnostics" / "timeseries.csv") as f:
        rows = list(csv.DictReader(f))
    cols = [str(c) for c in g["csv_cols"]]
    got = np.array([[float(r[c]) for c in cols] for r in rows])
    ref = g["csv_rows"]
    assert got.shape == ref.shape
    for j, c in enumerate(cols):
        a, b = got[:, j], ref[:, j]
        ok = ~np.isnan(b)
        assert np.array_equal(np.isnan(a), np.isnan(b)), c
        scale = max(np.abs(b[ok]).max() if ok.any() else 0.0, 1e-300)
        assert np.all(np.abs(a[ok] - b[ok]) <= 1e-10 * scale), (c, a, b)
