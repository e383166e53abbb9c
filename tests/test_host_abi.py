"""CPU-only checks: the C-ABI library loads and exports every declared
symbol, the ctypes table matches the header, and host-side geometry and
workload generators agree with the oracle."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from aeolus_gb300 import _lib, workloads
from aeolus_gb300.geodesic_grid import _ICO_F, _ICO_V, _subdivide_once
from aeolus_gb300.latlon_grid import fine_dims

HEADER = Path(__file__).resolve().parents[1] / "include" / "aeolus_gb300.h"


def header_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(aeolus_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_api():
    names = header_functions()
    assert "aeolus_synthesize" in names and "aeolus_swe_rk4" in names
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_library_exports_every_symbol():
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.aeolus_version() >= 10000


def test_bad_arguments_rejected_without_gpu():
    """Argument validation happens before any CUDA call."""
    import ctypes
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.aeolus_plan_create_gauss(1, 64, 10, 1.0, 0, ctypes.byref(h)) == _lib.ERR_ARG
    assert b"nlat >= 2" in lib.aeolus_last_error()
    assert lib.aeolus_spectral_op(9, 10, 1.0, None, None, 1, None) == _lib.ERR_ARG
    assert lib.aeolus_synthesize(None, None, None, 1, None, 0, None) == _lib.ERR_ARG
    with pytest.raises(ValueError):
        _lib.check(_lib.ERR_ARG)


@pytest.mark.parametrize("res", [0, 1, 2, 3])
def test_geodesic_point_order_matches_oracle(res):
    c, s = np.cos(1e-2), np.sin(1e-2)
    rot = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    v, f = _ICO_V @ rot.T, _ICO_F.copy()
    for _ in range(res):
        v, f = _subdivide_once(v, f)
    ov, of = oracle.geodesic.subdivide(res)
    np.testing.assert_array_equal(f, of)
    np.testing.assert_allclose(v, ov, rtol=0, atol=1e-15)
    assert len(v) == 10 * 4 ** res + 2


def test_fine_dims_rule():
    for nlat, nlon, L in [(32, 64, 21), (128, 256, 85), (192, 384, 127), (16, 32, 15), (160, 320, 106)]:
        assert fine_dims(nlat, nlon, L) == oracle.fine_dims(nlat, nlon, L)


def test_workload_generators():
    s, H = workloads.williamson2(21)
    o, Ho = oracle.models.williamson2(21, workloads.EARTH_RADIUS, workloads.EARTH_OMEGA)
    np.testing.assert_array_equal(s, o)
    assert H == Ho
    p, _ = workloads.perturbed_williamson2(21, seed=3)
    for f in range(3):
        ref = workloads.spectral_rms(s[f] if f != 1 else s[0])
        assert workloads.spectral_rms(p[f] - s[f]) == pytest.approx(0.01 * ref, rel=1e-12)
    z = workloads.bve_vorticity(21, 0)
    assert np.all(z[0] == 0) and np.all(z[:, 0].imag == 0)
    assert np.all(z[~workloads.triangle_mask(21)] == 0)
