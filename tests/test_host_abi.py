"""CPU-only checks: the C-ABI library loads and exports every declared
symbol, the ctypes table matches the header, and host-side geometry and
workload generators agree with the oracle."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from aeolus_gb300 import _lib, workloads
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


def test_geodesic_sizes_and_argument_checks():
    """Counts of the device geodesic build (host only) and its refusals
    before any launch."""
    lib = _lib.load()
    nv, nf, nb = ctypes.c_long(), ctypes.c_long(), ctypes.c_size_t()
    for r in range(0, 10):
        assert lib.aeolus_geodesic_sizes(r, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(nb)) == _lib.OK
        assert nv.value == 10 * 4 ** r + 2 and nf.value == 20 * 4 ** r
        assert nb.value >= 4 * 3 * nf.value * 3
        ov, of = oracle.geodesic.subdivide(min(r, 2)) if r <= 2 else (None, None)
        if ov is not None:
            assert (len(ov), len(of)) == (nv.value, nf.value)
    for bad in (-1, 10):
        assert lib.aeolus_geodesic_sizes(bad, None, None, None) == _lib.ERR_ARG
        assert b"resolution" in lib.aeolus_last_error()
    lib.aeolus_geodesic_sizes(3, None, None, ctypes.byref(nb))
    dummy = ctypes.c_void_p(16)  # never dereferenced: every call below is refused first
    assert lib.aeolus_geodesic_build(3, -1.0, *[dummy] * 7, dummy, nb.value, None) == _lib.ERR_ARG
    assert lib.aeolus_geodesic_build(3, 1.0, None, *[dummy] * 6, dummy, nb.value, None) == _lib.ERR_ARG
    assert lib.aeolus_geodesic_build(3, 1.0, *[dummy] * 7, dummy, nb.value - 1, None) == _lib.ERR_WORKSPACE


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


def test_sigma_grid_matches_oracle_and_rejects_bad_grids():
    from aeolus_gb300.primitive_equations import SigmaGrid, SigmaGridError
    from oracle import pe as ope
    for s in ([0.0, 1.0], [k / 7 for k in range(8)], [0.0, 0.05, 0.2, 0.5, 0.8, 1.0]):
        g, o = SigmaGrid(tuple(s)), ope.Sigma(s)
        assert g.nlev == o.K and g.thickness == tuple(o.dsig) and g.alpha == tuple(o.alpha)
        assert g.interface_log_ratios[1:] == tuple(o.beta[1:])
    assert SigmaGrid.uniform(4).interfaces == (0.0, 0.25, 0.5, 0.75, 1.0)
    for bad in ([0.1, 1.0], [0.0, 0.99], [0.0, 0.5, 0.5, 1.0], [0.0, float("nan"), 1.0], [0.0], ["a", 1.0]):
        with pytest.raises(SigmaGridError):
            SigmaGrid(tuple(bad))
    with pytest.raises(SigmaGridError):
        SigmaGrid.uniform(65)


def test_pe_entry_points_refuse_bad_arguments_without_gpu():
    lib = _lib.load()
    prm = _lib.PeParams(6.371e6, 7.292e-5, 287.04, 1004.64)
    sig = (ctypes.c_double * 3)(0.0, 0.5, 1.0)
    bad_sig = (ctypes.c_double * 3)(0.0, 0.5, 0.9)
    d = ctypes.c_void_p(16)  # never dereferenced: each call below is refused first
    assert lib.aeolus_pe_spectral(10, ctypes.byref(prm), 2, bad_sig, d, d, d, d, d, d, 1, None) == _lib.ERR_ARG
    assert b"sigma" in lib.aeolus_last_error()
    assert lib.aeolus_pe_spectral(10, ctypes.byref(prm), 0, sig, d, d, d, d, d, d, 1, None) == _lib.ERR_ARG
    assert lib.aeolus_pe_spectral(10, ctypes.byref(prm), 2, sig, None, d, d, d, d, d, 1, None) == _lib.ERR_ARG
    bad = _lib.PeParams(6.371e6, 7.292e-5, 287.04, 200.0)
    assert lib.aeolus_pe_spectral(10, ctypes.byref(bad), 2, sig, d, d, d, d, d, d, 1, None) == _lib.ERR_ARG
    assert b"cp_dry" in lib.aeolus_last_error()
    assert lib.aeolus_pe_derive(None, ctypes.byref(prm), 2, d, d, 1, None) == _lib.ERR_ARG
    assert lib.aeolus_pe_columns(None, ctypes.byref(prm), 2, sig, d, d, d, 1, None) == _lib.ERR_ARG
