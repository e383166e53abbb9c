"""Reference Gauss-Legendre rules at 50 significant digits (mpmath).

Writes tests/golden/gauss_exact.npz: for each n, the colatitudes (north ->
south), latitudes and weights rounded to float64.  Used to pin the device
Newton nodes/weights, which are more accurate than numpy.leggauss near the
poles (the reference's node source, latlon_grid.py:60).

Run:  python tests/golden/make_gauss_exact.py
"""
from pathlib import Path

import mpmath as mp
import numpy as np

NS = [2, 3, 16, 23, 32, 64, 96, 128, 160, 192]


def rule(n):
    mp.mp.dps = 50
    out_t, out_w = [], []
    for j in range((n + 1) // 2):
        if n % 2 and j == (n - 1) // 2:
            t = mp.pi / 2
        else:
            t = mp.pi * (j + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2)
            for _ in range(60):
                x = mp.cos(t)
                p0, p1 = mp.mpf(1), x
                for k in range(1, n):
                    p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
                dt = p1 * mp.sin(t) / (n * (x * p1 - p0))
                t -= dt
                if abs(dt) < mp.mpf(10) ** -45:
                    break
        x = mp.cos(t)
        p0, p1 = mp.mpf(1), x
        for k in range(1, n):
            p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
        q = n * (x * p1 - p0)
        out_t.append(t)
        out_w.append(2 * mp.sin(t) ** 2 / q ** 2)
    th = out_t + [mp.pi - t for t in reversed(out_t[: n // 2])]
    w = out_w + list(reversed(out_w[: n // 2]))
    lat = [mp.pi / 2 - t for t in th]
    return (np.array([float(v) for v in lat]), np.array([float(v) for v in w]))


def main():
    data = {}
    for n in NS:
        lat, w = rule(n)
        data[f"lat_{n}"] = lat
        data[f"w_{n}"] = w
    np.savez_compressed(Path(__file__).resolve().parent / "gauss_exact.npz", ns=np.array(NS), **data)


if __name__ == "__main__":
    main()
