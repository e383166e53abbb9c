"""GPU runs of ``aeolus run bve|swe`` against the reference's own runners.

The golden capsules (``tests/golden/run_*.npz``, made by
``tests/golden/make_golden.py runs``) are what the reference's ``run_swe`` /
``run_bve`` wrote for the same planets and initial states: the stored
coefficient snapshots, their times, and every diagnostics row.  The GB300
runner must store the same snapshots at bit-identical times, take the same
number of steps, match the coefficients to 1e-12 relative L2 and every
diagnostics column to 1e-10 of that column's scale (step lengths come from
the state-adaptive CFL ceiling, so they carry the FP64 round-off of the
characteristic speed).
"""
import numpy as np
import pytest
import torch

from helpers import rel_l2, tri

import aeolus_gb300 as ae
from aeolus_gb300 import runner as RN
from aeolus_gb300.shallow_water import ShallowWaterModel, ShallowWaterState, ShallowWaterStateError

pytestmark = pytest.mark.gpu
DEV = "cuda"
COEFF_TOL = 1e-12
ROW_TOL = 1e-10


def _read_csv(path):
    import csv
    with open(path) as f:
        rows = list(csv.DictReader(f))
    return list(rows[0].keys()), np.array([[float(r[c]) for c in rows[0]] for r in rows])


def _compare_rows(out_dir, g):
    cols, rows = _read_csv(out_dir / "diagnostics" / "timeseries.csv")
    assert cols == [str(c) for c in g["csv_cols"]]
    ref = g["csv_rows"]
    assert rows.shape == ref.shape
    for j, c in enumerate(cols):
        a, b = rows[:, j], ref[:, j]
        assert np.array_equal(np.isnan(a), np.isnan(b)), c
        ok = ~np.isnan(b)
        scale = max(np.abs(b[ok]).max() if ok.any() else 0.0, 1e-300)
        if c == "roundtrip_residual":
            scale = 1.0            # a ~1e-15 residual: compare absolutely
        assert np.all(np.abs(a[ok] - b[ok]) <= ROW_TOL * scale), (c, a, b)
    assert np.array_equal(rows[:, cols.index("step")], ref[:, cols.index("step")])


def _schedule(g):
    mode = str(g["mode"])
    if mode == "count":
        return dict(snapshot_mode="count", snapshot_times=list(g["snapshot_times"]), dt_snapshots=None)
    return dict(snapshot_mode="interval", dt_snapshots=float(g["dt_snapshots"]))


@pytest.mark.parametrize("name", ["run_swe_gauss32x64_L21_count", "run_swe_gauss16x32_L15_interval"])
def test_swe_run_matches_reference_runner(name, golden, tmp_path):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L, device=DEV)
    model = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]))
    state0 = ShallowWaterState(torch.as_tensor(g["state0"], device=DEV))
    RN.run_swe(model, state0, out_dir=tmp_path, t_end_days=float(g["t_end_days"]), plots=(), **_schedule(g))
    times = np.load(tmp_path / "swe_snapshot_times.npy")
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "swe_coeffs.npy")
    assert coeffs.shape == g["coeffs"].shape and coeffs.dtype == np.complex128
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= COEFF_TOL
    _compare_rows(tmp_path, g)


@pytest.mark.parametrize("name", ["run_bve_gauss32x64_L21_count", "run_bve_gauss16x32_L15_interval"])
def test_bve_run_matches_reference_runner(name, golden, tmp_path):
    g = golden(name)
    nlat, nlon, L = int(g["nlat"]), int(g["nlon"]), int(g["lmax"])
    planet = ae.make_planet("latlon", nlat=nlat, nlon=nlon, l_max=L, device=DEV)
    RN.run_bve(planet, g["zeta0"], out_dir=tmp_path, t_end_days=float(g["t_end_days"]),
               viscosity=float(g["nu"]), plots=(), **_schedule(g))
    times = np.load(tmp_path / RN.BVE_SNAPSHOT_TIMES_FILENAME)
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "vorticity_coeffs.npy")
    grid = np.load(tmp_path / "vorticity_grid.npy")
    assert coeffs.shape == g["coeffs"].shape and grid.shape == g["grid"].shape
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= COEFF_TOL
        assert rel_l2(grid[k], g["grid"][k]) <= COEFF_TOL
    _compare_rows(tmp_path, g)
    spec = np.load(tmp_path / "diagnostics" / "spectra.npz")
    # record times of intermediate steps accumulate CFL step lengths: not bitwise
    np.testing.assert_allclose(spec["times"], g["spec_times"], rtol=ROW_TOL, atol=0)
    assert rel_l2(spec["energy_l"], g["energy_l"]) <= COEFF_TOL
    assert rel_l2(spec["enstrophy_l"], g["enstrophy_l"]) <= COEFF_TOL


def test_swe_run_aborts_on_invalid_state_and_keeps_rows(tmp_path):
    """An invalid initial state is refused before any step; a state that
    turns invalid mid-run (NaN injected on the host into the step result of
    step 2) stops the run with ShallowWaterStateError naming the step, and
    the rows written before it stay on disk."""
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=10, device=DEV)
    model = ShallowWaterModel(planet, gravity=9.80616, mean_depth=10.0)
    bad = ShallowWaterState.zeros(10, device=DEV)
    bad.coeffs[2, 2, 0] = -1.0e4          # Phi0 + phi < 0 near the poles
    with pytest.raises(ShallowWaterStateError, match="initial state"):
        RN.run_swe(model, bad, dt_snapshots=600.0, t_end_days=0.01, out_dir=tmp_path, plots=())
    ok = ShallowWaterState.zeros(10, device=DEV)
    ok.coeffs[0, 3, 1] = 2e-5
    real_rk4, calls = model.rk4, []

    def faulty_rk4(coeffs, dt, nsteps=1, check=True):
        calls.append(dt)
        y = real_rk4(coeffs, dt, nsteps, check)
        return y * float("nan") if len(calls) == 2 else y

    model.rk4 = faulty_rk4
    with pytest.raises(ShallowWaterStateError, match=r"NaN/Inf.*\(step 2\)"):
        RN.run_swe(model, ok, dt_snapshots=3600.0, t_end_days=1.0, out_dir=tmp_path, plots=())
    cols, rows = _read_csv(tmp_path / "diagnostics" / "timeseries.csv")
    assert rows[:, cols.index("step")].tolist() == [0.0, 1.0]


def test_empty_count_schedule_writes_empty_stacks(tmp_path):
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=10, device=DEV)
    z = np.zeros((11, 11), complex)
    z[3, 1] = 1e-5
    RN.run_bve(planet, z, None, 0.05, tmp_path, 0.0, snapshot_times=[], snapshot_mode="count", plots=())
    assert np.load(tmp_path / "vorticity_coeffs.npy").shape == (0, 11, 11)
    assert np.load(tmp_path / "vorticity_grid.npy").shape[0] == 0
    assert np.load(tmp_path / RN.BVE_SNAPSHOT_TIMES_FILENAME).shape == (0,)


def test_bve_run_on_geodesic_fine_cogrid_matches_reference_runner(golden, tmp_path):
    """The reference's run_bve on a level-3 geodesic planet with the level-4
    product co-grid: the CFL ceiling comes from the minimum edge length."""
    g = golden("run_bve_geodesic_res3_L10_fine_count")
    planet = ae.make_planet("geodesic", resolution=int(g["res"]), l_max=int(g["lmax"]), product_quadrature="fine",
                            device=DEV)
    RN.run_bve(planet, g["zeta0"], out_dir=tmp_path, t_end_days=float(g["t_end_days"]), viscosity=float(g["nu"]),
               plots=(), **_schedule(g))
    times = np.load(tmp_path / RN.BVE_SNAPSHOT_TIMES_FILENAME)
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "vorticity_coeffs.npy")
    assert coeffs.shape == g["coeffs"].shape
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= COEFF_TOL
    _compare_rows(tmp_path, g)


def test_initial_conditions_match_reference(golden):
    """run/bve/initial_conditions.py and run/swe/initial_conditions.py on a
    Gauss 32x64 / l_max 21 planet, flat and over a mountain."""
    from aeolus_gb300 import initial_conditions as IC
    from aeolus_gb300.topography import Topography
    g = golden("ic_gauss32x64_L21")
    planet = ae.make_planet("latlon", nlat=32, nlon=64, l_max=21, device=DEV)
    for name in IC.INITIAL_CONDITIONS:
        z = IC.make_ic(name, planet)
        assert tuple(z.shape) == (32, 64) or name == "random_low_l"
        if name != "random_low_l":
            ref = g[f"bve_{name}"]
            assert np.abs(z.cpu().numpy() - ref).max() <= 1e-13 * np.abs(ref).max(), name
    topo = Topography.mountain(planet, height_m=1500.0, lat_deg=-20.0, lon_deg=45.0, width_deg=25.0)
    for tag, tp in (("flat", None), ("mountain", topo)):
        m = ShallowWaterModel(planet, gravity=float(g["gravity"]), mean_depth=float(g["mean_depth"]), topography=tp)
        for name in IC.SWE_INITIAL_CONDITIONS:
            st = IC.make_swe_ic(name, m).coeffs.cpu().numpy()
            ref = g[f"swe_{tag}_{name}"]
            assert rel_l2(tri(st), tri(ref)) <= COEFF_TOL if np.any(ref) else not np.any(st), (tag, name)
    with pytest.raises(ValueError, match="Unknown"):
        IC.make_ic("hurricane", planet)
    with pytest.raises(ValueError, match="Unknown"):
        IC.make_swe_ic("tsunami", m)


def test_pe_run_matches_reference_runner(golden, tmp_path):
    """The reference's fixed-step PE runner (run/pe/runner.py) on a thermal
    wave: stored states, times and every diagnostics row (the mass drift,
    a ~1e-13 round-off quantity, absolutely to 1e-12); and the balanced
    orographic rest state with its tendency."""
    from aeolus_gb300.initial_conditions import make_pe_ic
    from aeolus_gb300.primitive_equations import PrimitiveEquationsModel, SigmaGrid
    g = golden("run_pe_gauss16x32_L10_K3_thermal_wave")
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=int(g["lmax"]), device=DEV)
    model = PrimitiveEquationsModel(planet, SigmaGrid.uniform(int(g["nlev"])))
    st = make_pe_ic("thermal_wave", model, temperature=260.0, surface_pressure=1.0e5, thermal_amplitude=1.0)
    assert np.array_equal(st.coeffs.cpu().numpy(), g["state0"])
    RN.run_pe(model, st, dt_seconds=float(g["dt"]), t_end_days=float(g["t_end_days"]), out_dir=tmp_path,
              snapshot_times=list(g["snapshot_times"]), plots=())
    times = np.load(tmp_path / "pe_snapshot_times.npy")
    assert [t.hex() for t in times] == [t.hex() for t in g["times"]]
    coeffs = np.load(tmp_path / "pe_coeffs.npy")
    assert coeffs.shape == g["coeffs"].shape
    for k in range(coeffs.shape[0]):
        assert rel_l2(tri(coeffs[k]), tri(g["coeffs"][k])) <= COEFF_TOL
    cols, rows = _read_csv(tmp_path / "diagnostics" / "timeseries.csv")
    assert cols == [str(c) for c in g["csv_cols"]]
    ref = g["csv_rows"]
    assert rows.shape == ref.shape
    for j, c in enumerate(cols):
        a, b = rows[:, j], ref[:, j]
        assert np.array_equal(np.isnan(a), np.isnan(b)), c
        ok = ~np.isnan(b)
        tol = 1e-12 if c == "mass_rel_drift" else ROW_TOL * max(np.abs(b[ok]).max() if ok.any() else 0.0, 1e-300)
        assert np.all(np.abs(a[ok] - b[ok]) <= tol), (c, a, b)
    mo = PrimitiveEquationsModel(planet, SigmaGrid.uniform(int(g["nlev"])), surface_geopotential_lm=T(g["phi_s"]))
    oro = make_pe_ic("orographic_isothermal_rest", mo, temperature=260.0, surface_pressure=1.0e5)
    assert rel_l2(tri(oro.coeffs.cpu().numpy()), tri(g["oro_state"])) <= COEFF_TOL
    t = mo.tendency(oro.coeffs).cpu().numpy()
    assert np.abs(t).max() <= 1e-18 + 10 * np.abs(g["oro_tendency"]).max()


def test_pe_run_stage_fault_names_last_accepted_step(tmp_path):
    """A stage that fails validation during the second step is reported
    "in an RK4 stage after step 1", the last accepted step, as the reference
    runner does (run/pe/runner.py:93-106).  The fault is made on the host: the
    tendency turns non-finite from its fifth call on."""
    from aeolus_gb300.initial_conditions import make_pe_ic
    from aeolus_gb300.primitive_equations import (PrimitiveEquationsModel, PrimitiveEquationsStateError,
                                                  SigmaGrid)
    planet = ae.make_planet("latlon", nlat=16, nlon=32, l_max=10, device=DEV)
    model = PrimitiveEquationsModel(planet, SigmaGrid.uniform(3))
    st = make_pe_ic("thermal_wave", model, temperature=260.0, surface_pressure=1.0e5, thermal_amplitude=1.0)
    calls = [0]
    real = model.tendency

    def faulty(y):
        calls[0] += 1
        t = real(y)
        return t * float("nan") if calls[0] > 4 else t

    model.tendency = faulty
    with pytest.raises(PrimitiveEquationsStateError, match="in an RK4 stage after step 1"):
        RN.run_pe(model, st, dt_seconds=700.0, t_end_days=0.05, out_dir=tmp_path,
                  snapshot_times=[0.0, 2160.0, 4320.0], plots=())


def T(x):
    return torch.as_tensor(np.asarray(x), device=DEV)
