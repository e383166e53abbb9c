"""CPU oracle for the spectral hot path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy restatement of the reference's float64/complex128
algorithm (planetary_sandbox: dense point-set spherical-harmonic transform,
spectral operators, barotropic-vorticity and shallow-water tendencies, RK4,
conservation diagnostics, geodesic geometry).  Every function cites the
reference file:line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
(``cpu_baseline`` and ``--impl reference``) may import it, and only as the
checker or as the timed CPU baseline.  The product package ``aeolus_gb300``
never imports it and has no CPU fallback.

Parity pins: the restatement is checked against golden vectors produced by
running the reference's own Python and CUDA-C source on this CPU
(``tests/golden/make_golden.py``) and against ``scipy.special.sph_harm_y``.
The one deliberate difference from the reference: the associated-Legendre
basis uses the stable fully-normalised recurrence instead of the reference's
unnormalised recurrence times ``exp(lgamma(l-m+1) - lgamma(l+m+1))``
(src/planetary_sandbox/numerics/cuda/sh_matrix.cu:47-60), which underflows
for l + m >= ~175; below that the two agree to ~1e-13.
"""

from .sht import (  # noqa: F401
    gauss_latlon,
    legendre_table,
    dense_basis,
    PointSetSH,
    GaussSH,
    fine_dims,
    n_coeff,
)
from .operators import Operators  # noqa: F401
from . import models  # noqa: F401
from . import geodesic  # noqa: F401
from . import diagnostics  # noqa: F401
