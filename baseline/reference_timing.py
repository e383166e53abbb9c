"""Time the reference's own shallow-water tendency on the host cores.

The CPU baseline of ``bench.py``: the reference package (installed,
unmodified, into the git-ignored ``baseline/_ref/``) runs with the NumPy
stand-in for CuPy (``baseline/standin``), its CUDA-C basis kernel compiled
for the CPU by ``oracle/ref_build.py``.  The grid is the reference's own
``GaussLatLonGridGeometry`` (192 x 384); a bounded sample of its latitude
rows carries the reference's ``PointSetSphericalHarmonics`` (the dense basis
its Gauss transform uses, numerics/latlon_grid.py:151-199), and the
reference's ``ShallowWaterModel.tendency`` (physics/shallow_water.py:347-418)
is timed on it.  Its cost is linear in the point count (every transform is
a dense matrix-vector product over the points), so the bench scales the
sample to the full grid.  At l_max 127 the reference basis underflows for
l + m >= ~175: the results are not an oracle there, but the work is the
same.

Full steps, timed directly (no scaling):
* ``c1``: one barotropic-vorticity RK4 step (the reference's ``rk4_step``,
  run/bve/runner.py:211-216) on the Gauss 32 x 64 grid at l_max 21, the
  seeded vorticity spectrum ~N(0,1)(l+1)^-1.5 1e-5, dt 600 s, viscosity 0;
* ``c2``: one shallow-water RK4 step (the reference's ``rk4_step_array``,
  run/engine.py:406-431, over ``ShallowWaterModel.tendency``) on the Gauss
  128 x 256 grid at l_max 85 from a perturbed Williamson-2 state, dt 300 s.
Both build the reference's operator stack as its own tests do
(``GaussLatLonSphericalHarmonics`` + ``LatLonBackend`` with the "fine"
product space) and save the initial and final states to NPZ so that the
bench can compare its GPU step with the reference's own on the same inputs.

Run in its own process (the stand-in package is named ``cupy``):
    python baseline/reference_timing.py ROWS REPS
prints one JSON object {"seconds_per_tendency", "rows", "points", "modes"};
    python baseline/reference_timing.py c1|c2 REPS OUT.npz
prints {"config", "seconds_per_step", "reps", "setup_s", ...} and writes
OUT.npz (state0, state1).
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path
from types import SimpleNamespace

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
sys.dont_write_bytecode = True
sys.path[:0] = [str(HERE / "standin"), str(HERE / "_ref"), str(REPO)]

NLAT, NLON, LMAX = 192, 384, 127


def main(rows: int, reps: int) -> dict:
    import numpy as np
    from planetary_sandbox.numerics.latlon_grid import GaussLatLonGridGeometry
    from planetary_sandbox.numerics.fast_geodesic_sh import PointSetSphericalHarmonics
    from planetary_sandbox.numerics.spectral_operators import SpectralOperators
    from planetary_sandbox.physics.shallow_water import ShallowWaterModel

    from aeolus_gb300 import workloads as W

    R = W.EARTH_RADIUS
    grid = GaussLatLonGridGeometry(NLAT, NLON, R)
    lat = np.asarray(grid.point_latitudes).reshape(NLAT, NLON)
    lon = np.asarray(grid.point_longitudes).reshape(NLAT, NLON)
    w = np.asarray(grid.solid_angle_weights).reshape(NLAT, NLON)
    sel = np.linspace(0, NLAT - 1, rows).round().astype(int)
    plat, plon, pw = (a[sel].ravel() for a in (lat, lon, w))
    sh = PointSetSphericalHarmonics(plat, plon, LMAX, weights=pw)
    sample = SimpleNamespace(point_latitudes=plat, point_longitudes=plon, coslat=np.cos(plat),
                             cfl_length_scale=None)
    so = SpectralOperators(sh, R, sample, product_quadrature="coarse")
    planet = SimpleNamespace(sh=sh, so=so, grid=sample,
                             params=SimpleNamespace(radius=R, angular_velocity=W.EARTH_OMEGA))
    s0, depth = W.perturbed_williamson2(LMAX, seed=0)
    model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)
    model.tendency(s0.copy())  # warm-up
    t0 = time.perf_counter()
    for _ in range(reps):
        model.tendency(s0.copy())
    t = (time.perf_counter() - t0) / reps
    return {"seconds_per_tendency": t, "rows": rows, "points": int(plat.size),
            "modes": (LMAX + 1) * (LMAX + 2) // 2}


def full_step(config: str, reps: int, out: str) -> dict:
    """One full RK4 step of config c1 (BVE) or c2 (SWE), timed directly:
    median over `reps` steps from the same initial state after one untimed
    step."""
    import numpy as np
    from planetary_sandbox.numerics.latlon_grid import GaussLatLonGridGeometry, GaussLatLonSphericalHarmonics
    from planetary_sandbox.numerics.spherical_backend import LatLonBackend
    from planetary_sandbox.numerics.spectral_operators import SpectralOperators

    from aeolus_gb300 import workloads as W

    R = W.EARTH_RADIUS
    nlat, nlon, lmax, dt = {"c1": (32, 64, 21, 600.0), "c2": (128, 256, 85, 300.0)}[config]
    t0 = time.perf_counter()
    grid = GaussLatLonGridGeometry(nlat, nlon, R)
    sh = GaussLatLonSphericalHarmonics(grid, lmax)
    so = SpectralOperators(sh, R, grid, product_quadrature="fine", backend=LatLonBackend(grid, sh))
    planet = SimpleNamespace(sh=sh, so=so, grid=grid,
                             params=SimpleNamespace(radius=R, angular_velocity=W.EARTH_OMEGA))
    if config == "c1":
        from planetary_sandbox.physics.barotropic import BarotropicState, BarotropicVorticity
        from planetary_sandbox.run.bve.runner import rk4_step

        model = BarotropicVorticity(planet, viscosity=0.0)
        y0 = W.bve_vorticity(lmax, 0)

        def step():
            return rk4_step(model, BarotropicState(y0.copy()), 0.0, dt).coeffs
    else:
        from planetary_sandbox.physics.shallow_water import ShallowWaterModel
        from planetary_sandbox.run.engine import rk4_step_array

        y0, depth = W.perturbed_williamson2(lmax, seed=0)
        model = ShallowWaterModel(planet, gravity=W.GRAVITY, mean_depth=depth)

        def step():
            return rk4_step_array(model.tendency, y0.copy(), 0.0, dt)
    y1 = step()  # warm-up (also builds the product space)
    setup = time.perf_counter() - t0
    times = []
    for _ in range(max(reps, 1)):
        t1 = time.perf_counter()
        y1 = step()
        times.append(time.perf_counter() - t1)
    np.savez(out, state0=np.asarray(y0), state1=np.asarray(y1))
    times.sort()
    return {"config": config, "grid": f"gauss {nlat}x{nlon}", "l_max": lmax, "dt_s": dt,
            "seconds_per_step": times[len(times) // 2], "reps": len(times), "setup_s": setup}


if __name__ == "__main__":
    if sys.argv[1] in ("c1", "c2"):
        print(json.dumps(full_step(sys.argv[1], int(sys.argv[2]), sys.argv[3])))
    else:
        print(json.dumps(main(int(sys.argv[1]), int(sys.argv[2]))))
