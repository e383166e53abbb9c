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

Run in its own process (the stand-in package is named ``cupy``):
    python baseline/reference_timing.py ROWS REPS
prints one JSON object {"seconds_per_tendency", "rows", "points", "modes"}.
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


if __name__ == "__main__":
    print(json.dumps(main(int(sys.argv[1]), int(sys.argv[2]))))
