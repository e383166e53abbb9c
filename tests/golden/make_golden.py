"""Generate golden vectors by running the reference's own code on this CPU.

The reference (planetary_sandbox) is imported from its checkout with the
NumPy stand-in for CuPy in ``tests/golden/refshim``; its CUDA-C basis kernel
(src/planetary_sandbox/numerics/cuda/sh_matrix.cu) runs as C++ built by
``oracle/ref_build.py``.  Operators are built directly with a = 6.371e6 m and
Omega = 7.292e-5 1/s, as the workloads specify (``Planet.generate`` would
derive different constants and random terrain).

Run:  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [vector]
Writes ``tests/golden/*.npz`` (with ``vector``: only the weak-form curl/div
fixtures).  Only l_max <= 85 fixtures are made: above
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
REF_SRC = Path(os.environ.get("AEOLUS_REFERENCE_ROOT", "/root/reference")) / "src"
sys.dont_write_bytecode = True
sys.path[:0] = [str(HERE / "refshim"), str(REF_SRC), str(REPO)]

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


def geodesic_planet(res, lmax):
    grid = N.GeodesicGridGeometry(res, R)
    sh = N.GeodesicSphericalHarmonics(grid, lmax, weights="voronoi")
    backend = N.GeodesicBackend(grid, sh)
    so = N.SpectralOperators(sh, R, grid, product_quadrature="coarse", backend=backend)
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
    vector_cases()


if __name__ == "__main__":
    if sys.argv[1:] == ["vector"]:
        vector_cases()
    else:
        main()
