"""NumPy stand-in for CuPy, used only to run the reference on host cores.

Used by ``tests/golden/make_golden.py`` (golden vectors) and by the timed
CPU baseline (``baseline/reference_timing.py``): every ``cupy.X`` forwards to
``numpy.X``; ``RawModule`` runs the reference's own basis kernel compiled
for the CPU by ``oracle/ref_build.py``.
"""
import ctypes
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as _np

ndarray = _np.ndarray
random = _np.random
linalg = _np.linalg
fft = _np.fft


def __getattr__(name):
    return getattr(_np, name)


def is_available():
    return True


def asnumpy(a, *args, **kwargs):
    return _np.asarray(a)


def get_array_module(*args):
    return _np


class _Null:
    @staticmethod
    def synchronize():
        return None


cuda = SimpleNamespace(
    Stream=SimpleNamespace(null=_Null()),
    Device=lambda *a, **k: SimpleNamespace(synchronize=lambda: None,
                                            compute_capability="00"),
    runtime=SimpleNamespace(getDeviceCount=lambda: 1,
                            getDeviceProperties=lambda i: {"name": b"cpu-standin"},
                            runtimeGetVersion=lambda: 0,
                            driverGetVersion=lambda: 0),
)


def get_default_memory_pool():
    return SimpleNamespace(free_all_blocks=lambda: None, used_bytes=lambda: 0)


def get_default_pinned_memory_pool():
    return SimpleNamespace(free_all_blocks=lambda: None)


_REPO = Path(__file__).resolve().parents[3]
if str(_REPO) not in sys.path:
    sys.path.insert(0, str(_REPO))


class _BasisKernel:
    def __init__(self):
        from oracle import ref_build
        lib = ref_build.build()
        if lib is None:
            raise RuntimeError("reference checkout not found")
        self._lib = ctypes.CDLL(str(lib))
        self._fn = self._lib.launch_generate_sph_harm_basis
        self._fn.restype = None

    def __call__(self, grid, block, args):
        lat, lon, Y, n, l_max = args
        assert lat.dtype == _np.float64 and lon.dtype == _np.float64
        assert Y.dtype == _np.complex128 and Y.flags.c_contiguous
        lat = _np.ascontiguousarray(lat)
        lon = _np.ascontiguousarray(lon)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        self._fn(ctypes.c_uint(grid[0]), ctypes.c_uint(block[0]), p(lat), p(lon),
                 p(Y), ctypes.c_int(int(n)), ctypes.c_int(int(l_max)))


class RawModule:
    def __init__(self, code=None, **kwargs):
        self.code = code

    def get_function(self, name):
        if name == "generate_sph_harm_basis":
            return _BasisKernel()
        raise NotImplementedError(f"stand-in has no CPU build of kernel {name!r}")

    get_kernel = get_function


class RawKernel:
    def __init__(self, *a, **k):
        raise NotImplementedError("stand-in supports RawModule only")
