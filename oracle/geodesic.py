"""Oracle icosahedral geodesic point set (TEST INFRASTRUCTURE ONLY).

Restates src/planetary_sandbox/numerics/geodesic_grid.py:11-266 and the
"voronoi" weights of src/planetary_sandbox/numerics/optimized_geodesic_sh.py:127-133.
Point order must match the reference exactly (it fixes the row order of the
basis), so the subdivision visits faces and creates edge midpoints in the
same order as geodesic_grid.py:103-160.
"""
from __future__ import annotations

import numpy as np

_PHI = (1.0 + np.sqrt(5.0)) / 2.0
# Icosahedron vertices and faces, geodesic_grid.py:15-28.
ICO_VERTICES = np.array([
    [-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
    [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
    [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]]) / np.hypot(1, _PHI)
ICO_FACES = [
    [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
    [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
    [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
    [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]


def _rotate_x(v, angle=1e-2):
    """Anti-singularity rotation about x, geodesic_grid.py:37-38."""
    c, s = np.cos(angle), np.sin(angle)
    R = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    return v @ R.T


def subdivide(resolution: int):
    """Midpoint subdivision, geodesic_grid.py:103-160 (same visiting order)."""
    verts = [np.array(v) for v in _rotate_x(ICO_VERTICES)]
    faces = [list(f) for f in ICO_FACES]
    for _ in range(resolution):
        mid = {}
        new_faces = []

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            if key in mid:
                return mid[key]
            p = (verts[a] + verts[b]) / 2.0
            # normalize() of geodesic_grid.py:9: the axis form sums x*x + y*y
            # + z*z in order (the axis-free norm would go through a BLAS dot)
            verts.append(p / np.linalg.norm(p, axis=-1)[..., None])
            mid[key] = len(verts) - 1
            return mid[key]

        for v1, v2, v3 in faces:
            m12 = midpoint(v1, v2)
            m23 = midpoint(v2, v3)
            m31 = midpoint(v3, v1)
            new_faces += [[v1, m12, m31], [v2, m23, m12], [v3, m31, m23], [m12, m23, m31]]
        faces = new_faces
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.int64)


def latlon(points):
    """cartesian_to_spherical.py: lon in [-pi, pi], geocentric latitude."""
    x, y, z = points[:, 0], points[:, 1], points[:, 2]
    return np.arctan2(z, np.hypot(x, y)), np.arctan2(y, x)


def voronoi_areas(points, faces, radius: float = 1.0):
    """1/3 of each spherical triangle (L'Huilier), geodesic_grid.py:212-266."""
    n = points / np.linalg.norm(points, axis=1)[:, None]
    a, b, c = n[faces[:, 0]], n[faces[:, 1]], n[faces[:, 2]]
    dot = lambda u, v: np.clip(np.sum(u * v, axis=1), -1.0, 1.0)  # noqa: E731
    sa, sb, sc = np.arccos(dot(b, c)), np.arccos(dot(a, c)), np.arccos(dot(a, b))
    s = (sa + sb + sc) / 2.0
    t = np.sqrt(np.tan(s / 2) * np.tan((s - sa) / 2) * np.tan((s - sb) / 2)
                * np.tan((s - sc) / 2))
    area = 4.0 * np.arctan(t) * radius ** 2
    out = np.zeros(len(points))
    for k in range(3):  # same per-vertex accumulation as the reference loop
        np.add.at(out, faces[:, k], area / 3.0)
    return out


def geodesic_point_set(resolution: int, radius: float = 1.0):
    """(lat, lon, voronoi solid-angle weights summing to 4*pi)."""
    verts, faces = subdivide(resolution)
    pts = radius * verts
    lat, lon = latlon(pts)
    w = voronoi_areas(pts, faces, radius) / radius ** 2
    w = w * (4.0 * np.pi) / np.sum(w)
    return lat, lon, w
