"""The reference's own operator stack running on the GB300 transforms.

The unmodified reference package (``planetary_sandbox``, installed into the
git-ignored ``baseline/_ref``; NumPy in place of CuPy through the stand-in in
``baseline/standin``) is given the drop-in transform and backend objects of
``aeolus_gb300.dropin`` in place of its ``GaussLatLonSphericalHarmonics`` /
``LatLonBackend`` / ``GeodesicSphericalHarmonics``.  Its own
``SpectralOperators``, ``ShallowWaterModel``, ``BarotropicVorticity``,
``rk4_step_array``, ``rk4_step`` and ``run_swe`` then run with every
synthesis and analysis on the GPU, and their results must equal what the
reference produced with its own dense transforms (the golden vectors of
``tests/golden/make_golden.py``) to 1e-12 relative L2.

The reference package is imported into this process for the duration of the
module (its ``cupy`` is the NumPy stand-in) and removed afterwards; the tests
skip where it is not installed.
"""
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from helpers import rel_l2, tri

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
REF = ROOT / "baseline" / "_ref"
TOL = 1e-12
ROW_TOL = 1e-10


@pytest.fixture(scope="module")
def ref():
    if not (REF / "planetary_sandbox").is_dir():
        pytest.skip("the reference package is not installed in baseline/_ref")
    saved_path, saved_mods = list(sys.path), set(sys.modules)
    saved_bytecode = sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    sys.path[:0] = [str(ROOT / "baseline" / "standin"), str(REF)]
    try:
        import planetary_sandbox.numerics as N
        from planetary_sandbox.physics.barotropic import BarotropicState, BarotropicVorticity
        from planetary_sandbox.physics.shallow_water import ShallowWaterModel, ShallowWaterState
        from planetary_sandbox.run.bve.runner import rk4_step
        from planetary_sandbox.run.engine import rk4_step_array
        from planetary_sandbox.run.swe.runner import run_swe

        yield SimpleNamespace(N=N, BarotropicState=BarotropicState, BarotropicVorticity=BarotropicVorticity,
                              ShallowWaterModel=ShallowWaterModel, ShallowWaterState=ShallowWaterState,
                              rk4_step=rk4_step, rk4_step_array=rk4_step_array, run_swe=run_swe)
    finally:
        sys.path[:] = saved_path
        sys.dont_write_bytecode = saved_bytecode
        for name in set(sys.modules) - saved_mods:
            if name.split(".")[0] in ("cupy", "cupyx", "planetary_sandbox"):
                del sys.modules[name]


def gauss_planet(ref, g):
    """The reference's planet assembly (its geometry, SpectralOperators with
    the "fine" product quadrature) around the drop-in transform and backend."""
    from aeolus_gb300.dropin import GaussTransform, LatLonBackend
    R = float(g["radius"])
    grid = ref.N.GaussLatLonGridGeometry(int(g["nlat"]), int(g["nlon"]), R)
    sh = GaussTransform(grid, int(g["lmax"]))
    so = ref.N.SpectralOperators(sh, R, grid, product_quadrature="fine", backend=LatLonBackend(grid, sh))
    params = SimpleNamespace(radius=R, angular_velocity=float(g["omega"]))
    return SimpleNamespace(sh=sh, so=so, grid=grid, params=params)


def _uses_gb300(model):
    from aeolus_gb300.dropin import GaussTransform, PointSetTransform
    ps = model.so.backend.product_space(model.so.product_quadrature)
    return isinstance(model.sh, (GaussTransform, PointSetTransform)) and isinstance(
        ps.sh, (GaussTransform, PointSetTransform))


@pytest.mark.parametrize("name", ["swe_gauss32x64_L21", "swe_gauss16x32_L15_fine23x46", "swe_gauss128x256_L85"])
def test_reference_swe_model_on_gb300_transforms(ref, golden, name):
    """The reference's ShallowWaterModel.tendency and rk4_step_array
    (physics/shallow_water.py:347-418, run/engine.py:406-431), including a
    distinct 3/2-rule product grid (23x46) and config c2 (128x256, l_max 85)."""
    g = golden(name)
    planet = gauss_planet(ref, g)
    model = ref.ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    assert _uses_gb300(model)
    state = np.asarray(g["state"])
    assert rel_l2(tri(model.tendency(state.copy())), tri(g["tendency"])) <= TOL
    y = state.copy()
    for _ in range(int(g["steps"])):
        y = ref.rk4_step_array(model.tendency, y, 0.0, float(g["dt"]))
    assert rel_l2(tri(y), tri(g["rk4"])) <= TOL
    u, v = model.wind_on_state_grid(SimpleNamespace(coeffs=state))
    assert rel_l2(u, g["u"]) <= TOL and rel_l2(v, g["v"]) <= TOL
    ext = np.array(model.total_geopotential_extrema(SimpleNamespace(coeffs=state)))
    assert np.allclose(ext, g["phi_extrema"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", ["bve_gauss32x64_L21", "bve_gauss16x32_L15_fine23x46"])
def test_reference_bve_model_on_gb300_transforms(ref, golden, name):
    """The reference's BarotropicVorticity.tendency and its rk4_step
    (physics/barotropic.py:120-167, run/bve/runner.py:211-216), and the
    reference's round trip through the drop-in transform."""
    g = golden(name)
    planet = gauss_planet(ref, g)
    model = ref.BarotropicVorticity(planet, viscosity=float(g["nu"]))
    zeta = np.asarray(g["zeta"])
    grid_vals = planet.sh.inv_transform(zeta)
    assert isinstance(grid_vals, np.ndarray) and grid_vals.shape == (int(g["nlat"]) * int(g["nlon"]),)
    assert rel_l2(grid_vals, g["grid"]) <= TOL
    assert rel_l2(tri(planet.sh.transform(grid_vals)), tri(g["roundtrip"])) <= TOL
    tend = model.tendency(ref.BarotropicState(zeta.copy()), None)
    assert rel_l2(tri(tend), tri(g["tendency"])) <= TOL
    step = ref.rk4_step(model, ref.BarotropicState(zeta.copy()), 0.0, float(g["dt"])).coeffs
    assert rel_l2(tri(step), tri(g["rk4"])) <= TOL


def test_reference_run_swe_on_gb300_transforms(ref, golden, tmp_path):
    """The reference's own runner (run/swe/runner.py:29-150: snapshot
    scheduler, state-adaptive CFL, validation, diagnostics rows, capsule)
    over the drop-in transforms reproduces its own run capsule."""
    g = golden("run_swe_gauss32x64_L21_count")
    planet = gauss_planet(ref, g)
    model = ref.ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    ref.run_swe(model, ref.ShallowWaterState(np.array(g["state0"])), dt_snapshots=None,
                t_end_days=float(g["t_end_days"]), out_dir=tmp_path, snapshot_times=list(g["snapshot_times"]),
                plots=(), snapshot_mode="count")
    times = np.load(tmp_path / "swe_snapshot_times.npy")
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "swe_coeffs.npy")
    assert coeffs.shape == g["coeffs"].shape
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= TOL
    import csv
    with open(tmp_path / "diagnostics" / "timeseries.csv") as f:
        rows = list(csv.DictReader(f))
    cols = list(rows[0].keys())
    assert cols == [str(c) for c in g["csv_cols"]]
    got = np.array([[float(r[c]) for c in cols] for r in rows])
    want = g["csv_rows"]
    assert got.shape == want.shape
    for j, c in enumerate(cols):
        a, b = got[:, j], want[:, j]
        assert np.array_equal(np.isnan(a), np.isnan(b)), c
        ok = ~np.isnan(b)
        scale = 1.0 if c == "roundtrip_residual" else max(np.abs(b[ok]).max() if ok.any() else 0.0, 1e-300)
        assert np.all(np.abs(a[ok] - b[ok]) <= ROW_TOL * scale), c


def test_reference_geodesic_stack_on_gb300_point_set(ref, golden):
    """The reference's GeodesicBackend and SpectralOperators over a GB300
    point-set transform on its own level-3 icosahedral geometry with its own
    Voronoi weights (numerics/optimized_geodesic_sh.py:127-133): synthesis,
    analysis and the BVE tendency of the reference's golden vectors."""
    from aeolus_gb300.dropin import PointSetTransform
    g = golden("geodesic_res3_L10")
    R, L = float(g["radius"]), int(g["lmax"])
    grid = ref.N.GeodesicGridGeometry(int(g["res"]), R)
    weights = ref.N.GeodesicSphericalHarmonics(grid, L, weights="voronoi").weights
    sh = PointSetTransform(grid.point_latitudes, grid.point_longitudes, L, weights=weights)
    so = ref.N.SpectralOperators(sh, R, grid, product_quadrature="coarse", backend=ref.N.GeodesicBackend(grid, sh))
    planet = SimpleNamespace(sh=sh, so=so, grid=grid, params=SimpleNamespace(radius=R, angular_velocity=float(g["omega"])))
    assert rel_l2(sh.inv_transform(g["coeffs"]), g["synth"]) <= TOL
    assert rel_l2(tri(sh.transform(g["field"])), tri(g["analysis"])) <= TOL
    model = ref.BarotropicVorticity(planet, viscosity=0.0)
    assert _uses_gb300(model)
    tend = model.tendency(ref.BarotropicState(np.array(g["zeta"])), None)
    assert rel_l2(tri(tend), tri(g["bve_tendency"])) <= TOL


def test_dropin_backend_contract(ref):
    """Modes, caching, the "no silent fallback" error and describe() of the
    drop-in backend, as the reference's LatLonBackend gives them
    (numerics/spherical_backend.py:90-129, 170-211); the plan's Gauss nodes
    against the reference geometry's leggauss nodes."""
    from aeolus_gb300.dropin import GaussTransform, LatLonBackend
    grid = ref.N.GaussLatLonGridGeometry(16, 32, 6.371e6)
    sh = GaussTransform(grid, 15)
    be = LatLonBackend(grid, sh)
    theirs = ref.N.LatLonBackend(grid, ref.N.GaussLatLonSphericalHarmonics(grid, 15))
    assert be.supported_product_quadratures() == theirs.supported_product_quadratures()
    assert be.product_space("fine") is be.product_space("fine")
    assert be.product_space("coarse").sh is sh
    fine = be.product_space("fine")
    assert (fine.geometry.nlat, fine.geometry.nlon) == (23, 46) and fine.sh is not sh
    assert isinstance(fine.geometry, type(grid))
    with pytest.raises(ValueError, match="no silent fallback"):
        be.product_space("ultra")
    d, r = be.describe("fine"), theirs.describe("fine")
    assert {k: d[k] for k in d if k not in ("backend", "transform")} == {k: r[k] for k in r
                                                                        if k not in ("backend", "transform")}
    off = sh.node_offsets
    assert off["max_abs_latitude"] < 1e-14 and off["max_rel_weight"] < 1e-12
