"""Build recipe: compile the reference's basis kernel for the CPU (TEST INFRASTRUCTURE).

Compiles planetary_sandbox/numerics/cuda/sh_matrix.cu where it lies in the
reference package installed into the git-ignored baseline/_ref/ (or in the
reference checkout named by AEOLUS_REFERENCE_ROOT), as plain C++ with g++: a prelude header turns
``__global__`` into nothing and supplies ``blockIdx``/``blockDim``/
``threadIdx``; a stub ``cupy/complex.cuh`` maps ``complex<double>`` to
``std::complex<double>``; a generated launcher walks the launch grid.  The
output goes only to ``oracle/_ref/`` (git-ignored).  Nothing is copied from
the reference into the repository.

Used by ``tests/golden/make_golden.py`` (through the NumPy stand-in for CuPy)
and by the CPU-only pin tests when the reference source is present.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference package installed into the git-ignored baseline/_ref, or a
# reference checkout named by AEOLUS_REFERENCE_ROOT (its src/ tree)
_SRC = "planetary_sandbox/numerics/cuda/sh_matrix.cu"
SH_MATRIX = HERE.parent / "baseline" / "_ref" / _SRC
if os.environ.get("AEOLUS_REFERENCE_ROOT"):
    SH_MATRIX = Path(os.environ["AEOLUS_REFERENCE_ROOT"]) / "src" / _SRC
LIB = OUT / "libref_sh_matrix.so"

_PRELUDE = r"""
#include <math.h>
#include <cmath>
struct ref_dim3 { unsigned x, y, z; };
extern ref_dim3 blockIdx, blockDim, threadIdx, gridDim;
#define __global__
"""

_COMPLEX_STUB = r"""
#include <complex>
using std::complex;
"""

_LAUNCHER = r"""
#include <complex>
using std::complex;
struct ref_dim3 { unsigned x, y, z; };
ref_dim3 blockIdx, blockDim, threadIdx, gridDim;
extern "C" void generate_sph_harm_basis(const double*, const double*,
                                        complex<double>*, int, int);
extern "C" void launch_generate_sph_harm_basis(unsigned grid, unsigned block,
        const double* lat, const double* lon, complex<double>* Y, int n, int l_max) {
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned b = 0; b < grid; ++b)
        for (unsigned t = 0; t < block; ++t) {
            blockIdx = {b, 0, 0};
            threadIdx = {t, 0, 0};
            generate_sph_harm_basis(lat, lon, Y, n, l_max);
        }
}
"""


def available() -> bool:
    return SH_MATRIX.is_file()


def build(force: bool = False) -> Path | None:
    """Compile the reference basis kernel into oracle/_ref/; None if absent."""
    if not available():
        return None
    if LIB.exists() and not force and LIB.stat().st_mtime >= SH_MATRIX.stat().st_mtime:
        return LIB
    (OUT / "include" / "cupy").mkdir(parents=True, exist_ok=True)
    (OUT / "prelude.h").write_text(_PRELUDE)
    (OUT / "include" / "cupy" / "complex.cuh").write_text(_COMPLEX_STUB)
    (OUT / "launcher.cpp").write_text(_LAUNCHER)
    kobj = OUT / "sh_matrix.o"
    subprocess.run(["g++", "-O2", "-fPIC", "-std=c++17", "-c",
                    "-I", str(OUT / "include"), "-include", str(OUT / "prelude.h"),
                    "-x", "c++", str(SH_MATRIX), "-o", str(kobj)], check=True)
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-std=c++17",
                    str(OUT / "launcher.cpp"), str(kobj), "-o", str(LIB)], check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
