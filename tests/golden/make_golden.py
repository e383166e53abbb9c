"""Generate golden vectors by running the reference's own code on this CPU.

The reference (planetary_sandbox) is imported from its unmodified install in
the git-ignored baseline/_ref (or the checkout named by AEOLUS_REFERENCE_ROOT) with the
NumPy stand-in for CuPy in ``baseline/standin``; its CUDA-C basis kernel
(src/planetary_sandbox/numerics/cuda/sh_matrix.cu) runs as C++ built by
``oracle/ref_build.py``.  Operators are built directly with a = 6.371e6 m and
Omega = 7.292e-5 1/s, as the workloads specify (``Planet.generate`` would
derive different constants and random terrain).

Run:  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [vector|runs|geodesic_fine|pe|topo|ic|misc|pe_run]
Writes ``tests/golden/*.npz`` (with ``vector``: only the weak-form curl/div
fixtures; with ``runs``: only the integration-engine events and the run
capsules of the reference's BVE/SWE runners).  Only l_max <= 85 fixtures are made: above
that the reference basis kernel underflows (l + m >= ~175) and is not a
valid oracle.
"""
from __future__ import annotations

import os
import sys
import time
from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
# the reference package installed into the git-ignored baseline/_ref, or a
# reference checkout named by AEOLUS_REFERENCE_ROOT (its src/ tree)
REF_SRC = (Path(os.environ["AEOLUS_REFERENCE_ROOT"]) / "src" if os.environ.get("AEOLUS_REFERENCE_ROOT")
           else REPO / "baseline" / "_ref")
sys.dont_write_bytecode = True
sys.path[:0] = [str(REPO / "baseline" / "standin"), str(REF_SRC), str(REPO)]

import planetary_sandbox.numerics as N  # noqa: E402
from planetary_sandbox.physics.barotropic import BarotropicVorticity, BarotropicState  # noqa: E402
from planetary_sandbox.physics.shallow_water import ShallowWaterModel  # noqa: E402
from planetary_sandbox.run.engine import rk4_step_array  # noqa: E402
from planetary_sandbox.run.bve.runner import rk4_step  # noqa: E402
from planetary_sandbox.run.bve import diagnostics as bdiag  # noqa: E402

from aeolus_gb300 import workloads as W  # noqa: E402

R, OMEGA, G = W.EARTH_RADIUS, W.EARTH_OMEGA, W.GRAVITY


def latlon_planet(nlat, nlon, lmax, mode="fine"):
    grid = N.GaussLatLonGridGeometry(nlat, nlon, R)
    sh = N.GaussLatLonSphericalHarmonics(grid, lmax)
    backend = N.LatLonBackend(grid, sh)
    so = N.SpectralOperators(sh, R, grid, product_quadrature=mode, backend=backend)
    params = SimpleNamespace(radius=R, angular_velocity=OMEGA)
    return SimpleNamespace(sh=sh, so=so, grid=grid, params=params)


def geodesic_planet(res, lmax, mode="coarse"):
    grid = N.GeodesicGridGeometry(res, R)
    sh = N.GeodesicSphericalHarmonics(grid, lmax, weights="voronoi")
    backend = N.GeodesicBackend(grid, sh)
    so = N.SpectralOperators(sh, R, grid, product_quadrature=mode, backend=backend)
    params = SimpleNamespace(radius=R, angular_velocity=OMEGA)
    return SimpleNamespace(sh=sh, so=so, grid=grid, params=params)


def diag_arrays(d):
    keys = sorted(k for k, v in d.items() if np.isscalar(v))
    return np.array(keys), np.array([d[k] for k in keys], dtype=np.float64)


def bve_case(name, nlat, nlon, lmax, seed=0, dt=600.0, nu=0.0):
    t0 = time.time()
    p = latlon_planet(nlat, nlon, lmax)
    zeta = W.bve_vorticity(lmax, seed)
    model = BarotropicVorticity(p, viscosity=nu)
    grid_vals = p.sh.inv_transform(zeta)
    back = p.sh.transform(grid_vals)
    tend = model.tendency(BarotropicState(zeta.copy()), None)
    step = rk4_step(model, BarotropicState(zeta.copy()), 0.0, dt).coeffs
    sk0, sv0 = diag_arrays(bdiag.spectral_diagnostics(zeta, R, OMEGA))
    sk1, sv1 = diag_arrays(bdiag.spectral_diagnostics(step, R, OMEGA))
    gk0, gv0 = diag_arrays(bdiag.grid_diagnostics(zeta, p.sh, R, OMEGA,
                                                   p.grid.point_latitudes))
    psl = p.so.backend.product_space("fine")
    np.savez_compressed(
        HERE / f"{name}.npz", nlat=nlat, nlon=nlon, lmax=lmax, dt=dt, nu=nu,
        radius=R, omega=OMEGA, lat=np.asarray(p.grid.latitudes),
        weights=np.asarray(p.sh.weights), zeta=zeta, grid=grid_vals, roundtrip=back,
        tendency=tend, rk4=step, spec_keys=sk0, spec0=sv0, spec1=sv1,
        grid_keys=gk0, grid0=gv0,
        product_grid=np.array([psl.geometry.nlat, psl.geometry.nlon]))
    print(f"{name}: {time.time() - t0:.1f}s")


def swe_case(name, nlat, nlon, lmax, seed, dt, steps=1):
    t0 = time.time()
    p = latlon_planet(nlat, nlon, lmax)
    state, depth = W.perturbed_williamson2(lmax, seed)
    model = ShallowWaterModel(p, gravity=G, mean_depth=depth)
    tend = model.tendency(state.copy())
    y = state.copy()
    for _ in range(steps):
        y = rk4_step_array(model.tendency, y, 0.0, dt)
    psl = p.so.backend.product_space("fine")
    u, v = model.wind_on_state_grid(SimpleNamespace(coeffs=state))
    np.savez_compressed(
        HERE / f"{name}.npz", nlat=nlat, nlon=nlon, lmax=lmax, dt=dt, steps=steps,
        radius=R, omega=OMEGA, gravity=G, mean_depth=depth, state=state,
        tendency=tend, rk4=y, u=u, v=v,
        phi_extrema=np.array(model.total_geopotential_extrema(SimpleNamespace(coeffs=state))),
        product_grid=np.array([psl.geometry.nlat, psl.geometry.nlon]))
    print(f"{name}: {time.time() - t0:.1f}s")


def geodesic_case(name, res, lmax, seed=3):
    t0 = time.time()
    p = geodesic_planet(res, lmax)
    rng = np.random.default_rng(seed)
    a = W.random_spectrum(rng, lmax, -1.5, 1.0, zero_monopole=False)
    f = rng.standard_normal(p.grid.n_points)
    synth = p.sh.inv_transform(a)
    anal = p.sh.transform(f)
    zeta = W.bve_vorticity(lmax, seed)
    tend = BarotropicVorticity(p, viscosity=0.0).tendency(BarotropicState(zeta.copy()), None)
    np.savez_compressed(
        HERE / f"{name}.npz", res=res, lmax=lmax, radius=R, omega=OMEGA,
        lat=np.asarray(p.grid.latitudes), lon=np.asarray(p.grid.longitudes),
        weights=np.asarray(p.sh.weights), coeffs=a, synth=synth, field=f,
        analysis=anal, zeta=zeta, bve_tendency=tend)
    print(f"{name}: {time.time() - t0:.1f}s")


def vector_case(name, planet, seed):
    """Weak-form curl/div of a random tangent field on the product points
    (spectral_operators.py:399-492, truncate=True)."""
    t0 = time.time()
    so = planet.so
    ps = so._product_space
    lat = np.asarray(ps.sh.latitudes)
    rng = np.random.default_rng(seed)
    f_east = rng.standard_normal(lat.size)
    f_north = rng.standard_normal(lat.size)
    curl, div = so.vector_curl_div_spectral(f_east, f_north)
    np.savez_compressed(
        HERE / f"{name}.npz", lmax=so.l_max, radius=R, lat=lat, lon=np.asarray(ps.sh.longitudes),
        weights=np.asarray(ps.sh.weights), f_east=f_east, f_north=f_north, curl=np.asarray(curl),
        div=np.asarray(div))
    print(f"{name}: {time.time() - t0:.1f}s")


def geodesic_fine_case(name, res, lmax, seed=19, dt=600.0):
    """BVE and SWE on a geodesic planet whose product space is the reference's
    'fine' co-grid (resolution res+1, Voronoi weights)."""
    t0 = time.time()
    p = geodesic_planet(res, lmax, mode="fine")
    ps = p.so.backend.product_space("fine")
    zeta = W.bve_vorticity(lmax, seed)
    bve = BarotropicVorticity(p, viscosity=1e5)
    bve_t = bve.tendency(BarotropicState(zeta.copy()), None)
    bve_y = rk4_step(bve, BarotropicState(zeta.copy()), 0.0, dt).coeffs
    state, depth = W.perturbed_williamson2(lmax, seed + 1)
    swe = ShallowWaterModel(p, gravity=G, mean_depth=depth)
    swe_t = swe.tendency(state.copy())
    swe_y = rk4_step_array(swe.tendency, state.copy(), 0.0, dt)
    np.savez_compressed(
        HERE / f"{name}.npz", res=res, lmax=lmax, dt=dt, radius=R, omega=OMEGA, gravity=G, mean_depth=depth,
        fine_lat=np.asarray(ps.sh.latitudes), fine_lon=np.asarray(ps.sh.longitudes),
        fine_weights=np.asarray(ps.sh.weights), zeta=zeta, bve_tendency=bve_t, bve_rk4=bve_y,
        state=state, swe_tendency=swe_t, swe_rk4=swe_y,
        phi_extrema=np.array(swe.total_geopotential_extrema(SimpleNamespace(coeffs=state))),
        cfl_length_scale=np.float64(p.grid.cfl_length_scale))
    print(f"{name}: {time.time() - t0:.1f}s")


def topo_cases():
    """The reference's shallow-water model over a Gaussian mountain
    (physics/topography.py:207-292, shallow_water.py:226-271, :397-413):
    terrain coefficients, tendency and RK4 steps, with and without
    hyperdiffusion, and a run capsule of run_swe."""
    import tempfile
    from planetary_sandbox.physics.topography import Topography
    from planetary_sandbox.physics.shallow_water import ShallowWaterState
    from planetary_sandbox.run.swe.runner import run_swe
    from planetary_sandbox.run import engine as E
    t0 = time.time()
    nlat, nlon, L = 32, 64, 21
    p = latlon_planet(nlat, nlon, L)
    topo = Topography.mountain(p, height_m=2000.0, lat_deg=30.0, lon_deg=90.0, width_deg=20.0)
    state, depth = W.perturbed_williamson2(L, 29)
    out = {}
    for nu4 in (0.0, 1.0e16):
        m = ShallowWaterModel(p, gravity=G, mean_depth=depth, hyperdiffusion_nu4=nu4, topography=topo)
        key = "nu4" if nu4 else "plain"
        out[f"tendency_{key}"] = m.tendency(state.copy())
        y = state.copy()
        for _ in range(2):
            y = rk4_step_array(m.tendency, y, 0.0, 300.0)
        out[f"rk4_{key}"] = y
    m = ShallowWaterModel(p, gravity=G, mean_depth=depth, topography=topo)
    ext = m.surface_elevation_extrema
    with tempfile.TemporaryDirectory() as d:
        o = Path(d)
        times = E.count_snapshot_times(3, 0.05 * 86400.0)
        run_swe(m, ShallowWaterState(state.copy()), None, 0.05, o, snapshot_times=times, snapshot_mode="count",
                plots=())
        cols, rows = _csv_table(o / "diagnostics" / "timeseries.csv")
        np.savez_compressed(
            HERE / "topo_swe_gauss32x64_L21_mountain.npz", nlat=nlat, nlon=nlon, lmax=L, radius=R, omega=OMEGA,
            gravity=G, mean_depth=depth, nu4=1.0e16, dt=300.0, steps=2, height_m=2000.0, lat_deg=30.0,
            lon_deg=90.0, width_deg=20.0, elevation_lm=np.asarray(topo.elevation_lm), state=state,
            elevation_extrema=np.array(ext), t_end_days=0.05, snapshot_times=np.asarray(times, np.float64),
            coeffs=np.load(o / "swe_coeffs.npy"), times=np.load(o / "swe_snapshot_times.npy"), csv_cols=cols,
            csv_rows=rows, **out)
    print(f"topo_swe_gauss32x64_L21_mountain: {time.time() - t0:.1f}s")


def misc_cases():
    """The reference's scalar round-trip curl/div (numerics/spectral_operators.py:336-397)."""
    p = latlon_planet(16, 32, 15)
    ps = p.so.backend.product_space("fine")
    rng = np.random.default_rng(12)
    fe = rng.standard_normal(np.asarray(ps.sh.latitudes).size)
    fn = rng.standard_normal(fe.size)
    curl, div = p.so.vector_curl_div_roundtrip(fe, fn)
    np.savez_compressed(HERE / "misc_gauss16x32_L15.npz", f_east=fe, f_north=fn, rt_curl=np.asarray(curl),
                        rt_div=np.asarray(div))
    print("misc_gauss16x32_L15")


def pe_run_cases():
    """The reference's fixed-step PE runner (run/pe/runner.py) on a thermal
    wave, and its balanced orographic rest state (run/pe/initial_conditions.py)."""
    import tempfile
    from planetary_sandbox.physics.primitive_equations import PrimitiveEquationsModel
    from planetary_sandbox.physics.sigma_coordinate import SigmaGrid
    from planetary_sandbox.physics.topography import Topography
    from planetary_sandbox.run.pe.initial_conditions import make_pe_ic
    from planetary_sandbox.run.pe.runner import run_pe
    from planetary_sandbox.run import engine as E
    p = latlon_planet(16, 32, 10)
    model = PrimitiveEquationsModel(p, SigmaGrid.uniform(3))
    st = make_pe_ic("thermal_wave", model, temperature=260.0, surface_pressure=1.0e5, thermal_amplitude=1.0)
    topo = Topography.mountain(p, height_m=1000.0, lat_deg=20.0, lon_deg=60.0, width_deg=30.0, l_cut=6)
    mo = PrimitiveEquationsModel(p, SigmaGrid.uniform(3), surface_geopotential_lm=topo.surface_geopotential_lm(G))
    oro = make_pe_ic("orographic_isothermal_rest", mo, temperature=260.0, surface_pressure=1.0e5)
    with tempfile.TemporaryDirectory() as d:
        o = Path(d)
        times = E.count_snapshot_times(3, 0.05 * 86400.0)
        run_pe(model, st, dt_seconds=700.0, t_end_days=0.05, out_dir=o, snapshot_times=times, plots=())
        cols, rows = _csv_table(o / "diagnostics" / "timeseries.csv")
        np.savez_compressed(
            HERE / "run_pe_gauss16x32_L10_K3_thermal_wave.npz", lmax=10, nlev=3, radius=R, omega=OMEGA,
            state0=np.asarray(st.coeffs), dt=700.0, t_end_days=0.05, snapshot_times=np.asarray(times, np.float64),
            coeffs=np.load(o / "pe_coeffs.npy"), times=np.load(o / "pe_snapshot_times.npy"), csv_cols=cols,
            csv_rows=rows, phi_s=np.asarray(topo.surface_geopotential_lm(G)), oro_state=np.asarray(oro.coeffs),
            oro_tendency=np.asarray(mo.tendency(oro.coeffs.copy())))
    print("run_pe_gauss16x32_L10_K3_thermal_wave")


def ic_cases():
    """The reference's run initial conditions (run/bve/initial_conditions.py,
    run/swe/initial_conditions.py) on a Gauss 32x64 / l_max 21 planet, flat and
    over its mountain."""
    from planetary_sandbox.run.bve.initial_conditions import INITIAL_CONDITIONS, make_ic
    from planetary_sandbox.run.swe.initial_conditions import make_swe_ic
    from planetary_sandbox.physics.topography import Topography
    p = latlon_planet(32, 64, 21)
    out = {}
    for name in INITIAL_CONDITIONS:
        if name != "random_low_l":
            out[f"bve_{name}"] = np.asarray(make_ic(name, p))
    topo = Topography.mountain(p, height_m=1500.0, lat_deg=-20.0, lon_deg=45.0, width_deg=25.0)
    for tag, tp in (("flat", None), ("mountain", topo)):
        m = ShallowWaterModel(p, gravity=G, mean_depth=8000.0, topography=tp)
        for name in ("rest", "gravity_wave", "williamson2"):
            out[f"swe_{tag}_{name}"] = np.asarray(make_swe_ic(name, m).coeffs)
    np.savez_compressed(HERE / "ic_gauss32x64_L21.npz", nlat=32, nlon=64, lmax=21, radius=R, omega=OMEGA,
                        gravity=G, mean_depth=8000.0, elevation_lm=np.asarray(topo.elevation_lm), **out)
    print(f"ic_gauss32x64_L21: {len(out)} states")


def pe_state(lmax, nlev, seed, l_band=None, t0=260.0, ps0=101325.0):
    """Isothermal rest state plus seeded band-limited perturbations of every
    prognostic (the recipe of the reference's tests/test_pe_tendency.py:80-108)."""
    n = lmax + 1
    l_band = (2 * lmax) // 3 if l_band is None else l_band
    rng = np.random.default_rng(seed)
    s = np.zeros((3 * nlev + 1, n, n), complex)
    s[2 * nlev:3 * nlev, 0, 0] = t0 * np.sqrt(4 * np.pi)
    s[3 * nlev, 0, 0] = np.log(ps0) * np.sqrt(4 * np.pi)

    def pert(amp, zero_monopole):
        p = amp * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        p[:, 0] = p[:, 0].real
        p *= np.tril(np.ones((n, n)))
        p[l_band + 1:, :] = 0.0
        if zero_monopole:
            p[0, 0] = 0.0
        return p

    for k in range(nlev):
        s[k] += pert(2e-6, True)
        s[nlev + k] += pert(2e-6, True)
        s[2 * nlev + k] += pert(0.5, False)
    s[3 * nlev] += pert(1e-3, True)
    return s


def pe_case(name, planet, interfaces, seed, phi_s_amp=0.0):
    """The reference's dry hydrostatic primitive-equation tendency
    (physics/primitive_equations.py:727-753) on a seeded state."""
    from planetary_sandbox.physics.primitive_equations import PrimitiveEquationsModel
    from planetary_sandbox.physics.sigma_coordinate import SigmaGrid
    t0 = time.time()
    L = planet.sh.l_max
    sigma = SigmaGrid(tuple(interfaces))
    phi_s = None
    if phi_s_amp:
        rng = np.random.default_rng(seed + 100)
        cut = (2 * L) // 3
        phi_s = np.zeros((L + 1, L + 1), complex)
        phi_s[:cut + 1, :cut + 1] = phi_s_amp * (rng.standard_normal((cut + 1, cut + 1))
                                                 + 1j * rng.standard_normal((cut + 1, cut + 1)))
        phi_s[:, 0] = phi_s[:, 0].real
        phi_s *= np.tril(np.ones((L + 1, L + 1)))
    model = PrimitiveEquationsModel(planet, sigma, surface_geopotential_lm=phi_s)
    state = pe_state(L, sigma.nlev, seed)
    tend = model.tendency(state.copy())
    np.savez_compressed(
        HERE / f"{name}.npz", lmax=L, interfaces=np.asarray(interfaces, float), radius=R, omega=OMEGA,
        r_dry=model.r_dry, cp_dry=model.cp_dry,
        phi_s=np.zeros((L + 1, L + 1), complex) if phi_s is None else phi_s, state=state, tendency=tend)
    print(f"{name}: {time.time() - t0:.1f}s")


def pe_cases():
    pe_case("pe_gauss16x32_L15_fine23x46_K5", latlon_planet(16, 32, 15), [k / 5 for k in range(6)], seed=31)
    pe_case("pe_gauss24x48_L15_K4_nonuniform_phis", latlon_planet(24, 48, 15), [0.0, 0.12, 0.35, 0.7, 1.0],
            seed=37, phi_s_amp=300.0)
    pe_case("pe_geodesic_res3_L10_K3", geodesic_planet(3, 10), [0.0, 0.3, 0.65, 1.0], seed=41)


def vector_cases():
    vector_case("vector_gauss16x32_L15_fine23x46", latlon_planet(16, 32, 15), seed=13)
    vector_case("vector_geodesic_res3_L10", geodesic_planet(3, 10), seed=17)


def main():
    # Small BVE workload: Gauss 32x64, l_max=21, one RK4 step at dt=600 s.
    bve_case("bve_gauss32x64_L21", 32, 64, 21)
    # Distinct 3/2-rule product grid (23x46: odd rows, length-46 longitudes).
    bve_case("bve_gauss16x32_L15_fine23x46", 16, 32, 15, seed=5, dt=900.0, nu=1e5)
    swe_case("swe_gauss16x32_L15_fine23x46", 16, 32, 15, seed=7, dt=300.0)
    swe_case("swe_gauss32x64_L21", 32, 64, 21, seed=11, dt=300.0, steps=2)
    # Shallow-water workload grid: Gauss 128x256, l_max=85.
    swe_case("swe_gauss128x256_L85", 128, 256, 85, seed=2, dt=300.0)
    geodesic_case("geodesic_res3_L10", 3, 10)
    geodesic_fine_case("geodesic_fine_res3_L10", 3, 10)
    pe_cases()
    topo_cases()
    ic_cases()
    misc_cases()
    pe_run_cases()
    vector_cases()


# ----------------------------------------------------------- run driver
def _events_hex(events):
    return [[k, float(dt).hex(), float(t).hex()] for k, dt, t in events]


def _outcome(fn, *a, **kw):
    try:
        return {"value": float(fn(*a, **kw)).hex()}
    except Exception as exc:  # the reference's error contract is part of the pin
        return {"raises": type(exc).__name__}


def schedule_cases():
    """Events of the reference's IntegrationScheduler (engine.py) for fixed and
    state-adaptive ceilings, plus its schedule and CFL helpers' outcomes."""
    import json
    from planetary_sandbox.run import engine as E

    cases = []

    def plan(name, t_end, dt_cfl, **kw):
        cases.append({"name": name, "kind": "plan", "t_end": t_end, "dt_cfl": dt_cfl, "kw": kw,
                      "events": _events_hex(E.integration_plan(t_end, dt_cfl, **kw))})

    plan("count_aligned", 3600.0, 600.0, mode="count", snapshot_times=E.count_snapshot_times(4, 3600.0))
    plan("count_nonaligned", 1000.0, 300.0, mode="count", snapshot_times=E.count_snapshot_times(3, 1000.0))
    plan("count_one", 1234.5, 500.0, mode="count", snapshot_times=E.count_snapshot_times(1, 1234.5))
    plan("count_empty", 900.0, 400.0, mode="count", snapshot_times=[])
    plan("count_thirds", 86400.0 / 3, 977.0, mode="count", snapshot_times=E.count_snapshot_times(7, 86400.0 / 3))
    plan("interval_aligned", 3600.0, 500.0, mode="interval", dt_snapshots=1200.0)
    plan("interval_nonaligned", 8640.0, 700.0, mode="interval", dt_snapshots=5000.0)
    plan("interval_tolerance", 3600.0 + 1e-4, 450.0, mode="interval", dt_snapshots=900.0)
    plan("interval_big_ceiling", 1000.0, 1e6, mode="interval", dt_snapshots=300.0)

    def adaptive(name, t_end, speeds, length_scale, **kw):
        sch = E.IntegrationScheduler(t_end, **kw)
        events = []

        def on_store(t):
            events.append(("store", 0.0, t))

        def on_step(t0, t1, dt, k):
            events.append(("step", dt, t1))
            return speeds[(k - 1) % len(speeds)]

        dt0 = E.advective_cfl_timestep(length_scale, speeds[-1])
        out = E.integrate(sch, dt0, length_scale, on_step=on_step, on_store=on_store)
        cases.append({"name": name, "kind": "adaptive", "t_end": t_end, "speeds": speeds,
                      "length_scale": length_scale, "kw": kw, "events": _events_hex(events),
                      "final": [float(out[0]).hex(), out[1]]})

    adaptive("adaptive_count", 7200.0, [35.0, 80.0, 20.0, 55.5], 6.2e5 / 4,
             mode="count", snapshot_times=E.count_snapshot_times(5, 7200.0))
    adaptive("adaptive_interval", 7200.0, [120.0, 300.0, 75.0], 2.0e5,
             mode="interval", dt_snapshots=2500.0)
    adaptive("adaptive_motionless", 2000.0, [0.0], 1.0e5, mode="count", snapshot_times=[0.0, 2000.0])
    adaptive("adaptive_no_length_scale", 2000.0, [10.0], None, mode="interval", dt_snapshots=1000.0)

    # A ceiling below one ulp of t cannot advance the clock: the planner raises.
    sch = E.IntegrationScheduler(1.0e6, mode="count", snapshot_times=[5.0e5, 1.0e6])
    seq = [5.0e5, 1e-12]
    got = []
    try:
        for dt in [seq[0]] + [seq[1]] * 4:
            got.append(sch.next_event(dt))
        stagnation = "none"
    except Exception as exc:
        stagnation = type(exc).__name__
    cases.append({"name": "count_stagnation", "kind": "stagnation", "raises": stagnation,
                  "events": _events_hex([e for e in got if e is not None])})

    helpers = {
        "cfl": [[ls, sp, _outcome(E.advective_cfl_timestep, ls, sp)] for ls, sp in
                [(6.2e5, 40.0), (None, 40.0), (0.0, 40.0), (6.2e5, 0.0), (1.0, 1e-300), (-1.0, 3.0),
                 (6.2e5, -1.0), (6.2e5, float("nan")), (float("inf"), 3.0), (1e308, 1e-300)]],
        "validate": [],
        "interval_times": [[d, t, [float(x).hex() for x in E.interval_snapshot_times(d, t)]]
                           for d, t in [(600.0, 3600.0), (700.0, 3600.0), (900.0, 3600.0 + 1e-4),
                                        (1000.0, 999.9)]],
        "count_times": [[n, t, [float(x).hex() for x in E.count_snapshot_times(n, t)]]
                        for n, t in [(0, 100.0), (1, 100.0), (2, 100.0), (7, 86400.0 / 3)]],
    }
    for times, t_end in [([0.0, 50.0, 100.0], 100.0), ([-1e-8, 100.0 + 1e-8], 100.0), ([0.0, 0.0], 100.0),
                         ([10.0, 5.0], 100.0), ([-1.0], 100.0), ([101.0], 100.0), ([float("nan")], 100.0),
                         ([1.0], 0.0), ([1.0], float("inf"))]:
        try:
            helpers["validate"].append([times, t_end, {"value": [float(x).hex() for x in
                                                                 E.validate_snapshot_schedule(times, t_end)]}])
        except Exception as exc:
            helpers["validate"].append([times, t_end, {"raises": type(exc).__name__}])
    for bad in [float("nan"), 0.0, -5.0]:
        try:
            E.IntegrationScheduler(100.0, mode="count", snapshot_times=[100.0]).next_event(bad)
            helpers.setdefault("bad_ceiling", []).append([bad, "none"])
        except Exception as exc:
            helpers.setdefault("bad_ceiling", []).append([bad, type(exc).__name__])
    with open(HERE / "schedule_events.json", "w") as f:
        json.dump({"source": "planetary_sandbox.run.engine (reference), made by make_golden.py runs",
                   "cases": cases, "helpers": helpers}, f, indent=0, allow_nan=True)
    print(f"schedule_events.json: {len(cases)} cases")


def _csv_table(path):
    import csv
    with open(path) as f:
        rows = list(csv.DictReader(f))
    cols = list(rows[0].keys())
    return np.array(cols), np.array([[float(r[c]) for c in cols] for r in rows], dtype=np.float64)


def run_cases():
    """The reference's own run_swe / run_bve (no figures) on small Gauss
    planets, in count and interval mode; their capsule arrays and CSV rows."""
    import tempfile
    from planetary_sandbox.physics.shallow_water import ShallowWaterState
    from planetary_sandbox.run.swe.runner import run_swe
    from planetary_sandbox.run.bve.runner import run_bve

    def swe(name, nlat, nlon, lmax, seed, t_end_days, **kw):
        t0 = time.time()
        p = latlon_planet(nlat, nlon, lmax)
        state, depth = W.perturbed_williamson2(lmax, seed)
        model = ShallowWaterModel(p, gravity=G, mean_depth=depth)
        with tempfile.TemporaryDirectory() as d:
            out = Path(d)
            run_swe(model, ShallowWaterState(state.copy()), out_dir=out, t_end_days=t_end_days, plots=(), **kw)
            cols, rows = _csv_table(out / "diagnostics" / "timeseries.csv")
            np.savez_compressed(
                HERE / f"{name}.npz", nlat=nlat, nlon=nlon, lmax=lmax, radius=R, omega=OMEGA, gravity=G,
                mean_depth=depth, state0=state, t_end_days=t_end_days,
                mode=kw["snapshot_mode"], snapshot_times=np.asarray(kw.get("snapshot_times") or [], np.float64),
                dt_snapshots=np.float64(kw.get("dt_snapshots") or 0.0),
                coeffs=np.load(out / "swe_coeffs.npy"), times=np.load(out / "swe_snapshot_times.npy"),
                csv_cols=cols, csv_rows=rows)
        print(f"{name}: {time.time() - t0:.1f}s, {rows.shape[0]} rows")

    def bve(name, nlat, nlon, lmax, seed, nu, t_end_days, **kw):
        t0 = time.time()
        p = latlon_planet(nlat, nlon, lmax)
        zeta = W.bve_vorticity(lmax, seed)
        with tempfile.TemporaryDirectory() as d:
            out = Path(d)
            run_bve(p, zeta.copy(), out_dir=out, t_end_days=t_end_days, viscosity=nu, plots=(), **kw)
            cols, rows = _csv_table(out / "diagnostics" / "timeseries.csv")
            spec = np.load(out / "diagnostics" / "spectra.npz")
            np.savez_compressed(
                HERE / f"{name}.npz", nlat=nlat, nlon=nlon, lmax=lmax, radius=R, omega=OMEGA, nu=nu,
                zeta0=zeta, t_end_days=t_end_days, mode=kw["snapshot_mode"],
                snapshot_times=np.asarray(kw.get("snapshot_times") or [], np.float64),
                dt_snapshots=np.float64(kw.get("dt_snapshots") or 0.0),
                coeffs=np.load(out / "vorticity_coeffs.npy"), grid=np.load(out / "vorticity_grid.npy"),
                times=np.load(out / "bve_snapshot_times.npy"), csv_cols=cols, csv_rows=rows,
                spec_times=spec["times"], energy_l=spec["energy_l"], enstrophy_l=spec["enstrophy_l"])
        print(f"{name}: {time.time() - t0:.1f}s, {rows.shape[0]} rows")

    from planetary_sandbox.run import engine as E
    t_end = 0.08
    swe("run_swe_gauss32x64_L21_count", 32, 64, 21, 21, t_end, dt_snapshots=None,
        snapshot_times=E.count_snapshot_times(4, t_end * 86400.0), snapshot_mode="count")
    swe("run_swe_gauss16x32_L15_interval", 16, 32, 15, 23, 0.1, dt_snapshots=5000.0, snapshot_mode="interval")
    bve("run_bve_gauss32x64_L21_count", 32, 64, 21, 0, 1e5, 3.0, dt_snapshots=None,
        snapshot_times=E.count_snapshot_times(3, 3.0 * 86400.0), snapshot_mode="count")
    bve("run_bve_gauss16x32_L15_interval", 16, 32, 15, 4, 0.0, 1.5, dt_snapshots=40000.0,
        snapshot_mode="interval")

    # geodesic planet with the res r+1 product co-grid: CFL from the minimum edge length
    t0 = time.time()
    p = geodesic_planet(3, 10, mode="fine")
    zeta = W.bve_vorticity(10, 6)
    with tempfile.TemporaryDirectory() as d:
        out = Path(d)
        times = E.count_snapshot_times(3, 1.0 * 86400.0)
        run_bve(p, zeta.copy(), None, 1.0, out, 1e5, snapshot_times=times, snapshot_mode="count", plots=())
        cols, rows = _csv_table(out / "diagnostics" / "timeseries.csv")
        spec = np.load(out / "diagnostics" / "spectra.npz")
        np.savez_compressed(
            HERE / "run_bve_geodesic_res3_L10_fine_count.npz", res=3, lmax=10, radius=R, omega=OMEGA, nu=1e5,
            zeta0=zeta, t_end_days=1.0, mode="count", snapshot_times=np.asarray(times, np.float64),
            dt_snapshots=np.float64(0.0), coeffs=np.load(out / "vorticity_coeffs.npy"),
            grid=np.load(out / "vorticity_grid.npy"), times=np.load(out / "bve_snapshot_times.npy"),
            csv_cols=cols, csv_rows=rows, spec_times=spec["times"], energy_l=spec["energy_l"],
            enstrophy_l=spec["enstrophy_l"])
    print(f"run_bve_geodesic_res3_L10_fine_count: {time.time() - t0:.1f}s, {rows.shape[0]} rows")


if __name__ == "__main__":
    if sys.argv[1:] == ["vector"]:
        vector_cases()
    elif sys.argv[1:] == ["topo"]:
        topo_cases()
    elif sys.argv[1:] == ["ic"]:
        ic_cases()
    elif sys.argv[1:] == ["pe_run"]:
        pe_run_cases()
    elif sys.argv[1:] == ["misc"]:
        misc_cases()
    elif sys.argv[1:] == ["pe"]:
        pe_cases()
    elif sys.argv[1:] == ["geodesic_fine"]:
        geodesic_fine_case("geodesic_fine_res3_L10", 3, 10)
    elif sys.argv[1:] == ["runs"]:
        schedule_cases()
        run_cases()
    else:
        main()
