"""Device-built geodesic point sets against the oracle's restatement of the
reference construction (src/planetary_sandbox/numerics/geodesic_grid.py).

Faces must be identical (the point order fixes the rows of every basis);
midpoints are rounded like the reference's, so points differ only by the
last bits of the icosahedron seed (the host's cos/sin of the 1e-2 rad
rotation; checked to 1e-15 of the radius); coordinates use CUDA's
atan2/hypot (a few ulp).  Areas follow the reference's L'Huilier form,
whose sides are acos of near-unit dot products: the last-bit differences
between CUDA's and the host's acos/tan/atan grow like 1/side^2 there (4e-13
relative at resolution 5), so areas are checked to 5e-12 relative and their
sum to 1e-12 of 4 pi R^2; the transforms built on them are checked against
the reference's golden vectors in the parity tests.
"""
import time

import numpy as np
import pytest
import torch

import oracle
from aeolus_gb300.ops import geodesic_build
from aeolus_gb300.geodesic_grid import GeodesicGridGeometry

pytestmark = pytest.mark.gpu
R = 6.371e6


def _oracle_min_edge(points, faces):
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    d = np.sqrt(np.sum((points[e[:, 0]] - points[e[:, 1]]) ** 2, axis=1))
    return d[d > 0].min()


@pytest.mark.parametrize("res", [0, 1, 2, 3, 4, 5, 6])
def test_device_geodesic_matches_oracle(res):
    g = geodesic_build(res, R, "cuda")
    ov, of = oracle.geodesic.subdivide(res)
    op = R * ov
    np.testing.assert_array_equal(g["faces"].cpu().numpy(), of)
    pts = g["points"].cpu().numpy()
    np.testing.assert_allclose(pts, op, rtol=0, atol=1e-15 * R)
    lat, lon = oracle.geodesic.latlon(op)
    np.testing.assert_allclose(g["lat"].cpu().numpy(), lat, rtol=0, atol=2e-15)
    np.testing.assert_allclose(g["lon"].cpu().numpy(), lon, rtol=0, atol=4e-15)
    areas = oracle.geodesic.voronoi_areas(op, of, R)
    np.testing.assert_allclose(g["areas"].cpu().numpy(), areas, rtol=5e-12)
    assert g["min_edge"] == pytest.approx(_oracle_min_edge(op, of), rel=1e-14)
    assert abs(g["areas"].sum().item() / (4 * np.pi * R ** 2) - 1.0) < 1e-12


def test_geometry_class_uses_device_build_and_is_repeatable():
    a = GeodesicGridGeometry(4, R, "cuda")
    b = GeodesicGridGeometry(4, R, "cuda")
    assert torch.equal(a.cell_areas, b.cell_areas) and torch.equal(a.latitudes, b.latitudes)
    assert a.latitudes.is_cuda and a.cell_areas.is_cuda
    assert a.points.shape == (2562, 3) and a.faces.shape == (5120, 3)
    assert a.cfl_length_scale == pytest.approx(_oracle_min_edge(a.points, a.faces.astype(np.int64)), rel=1e-15)


def test_level8_build_time_and_counts():
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = geodesic_build(8, R, "cuda")
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert g["points"].shape == (655362, 3)
    # every vertex has 5 (the 12 icosahedron corners) or 6 incident faces
    counts = torch.bincount(g["faces"].reshape(-1).long(), minlength=655362)
    assert int((counts == 5).sum()) == 12 and int((counts == 6).sum()) == 655362 - 12
    print(f"geodesic level 8 built on the device in {dt * 1e3:.1f} ms")
