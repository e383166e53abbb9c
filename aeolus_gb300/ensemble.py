"""Batched uneven ensembles: BVE members of different l_max advanced together.

Each group is a :class:`~aeolus_gb300.barotropic.BarotropicVorticity` model
(its own Gauss grid and product-space plan) with a batch of members; every
RK4 stage launches each stage kernel once for all groups
(``aeolus_ensemble_bve_rk4``), a whole step can be captured into a CUDA graph
and replayed (``aeolus_ensemble_capture`` / ``aeolus_ensemble_launch``), and
``autotune`` times candidate launch shapes per group on the ensemble's own
states (``aeolus_ensemble_autotune``).

The reference runs one state per process (run/bve/runner.py:211-216); the
per-member arithmetic here is that of ``BarotropicVorticity.rk4``.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int, c_size_t, c_void_p

import torch

from . import _lib
from ._lib import check
from .ops import _stream


class BarotropicEnsemble:
    def __init__(self, models, batches):
        if len(models) != len(batches) or not models:
            raise ValueError("need one batch size per model")
        self.models = list(models)
        self.batches = [int(b) for b in batches]
        self.device = self.models[0].f_lm.device
        lib = _lib.load()
        n = len(models)
        plans = (c_void_p * n)(*[m._plan.handle.value for m in self.models])
        bs = (c_int * n)(*self.batches)
        prm = (_lib.BveParams * n)(*[_lib.BveParams(m.R, m.Omega, m.nu) for m in self.models])
        self.handle = c_void_p()
        check(lib.aeolus_ensemble_create(n, ctypes.cast(plans, ctypes.POINTER(c_void_p)), bs, prm,
                                         byref(self.handle)))
        nbytes = c_size_t()
        check(lib.aeolus_ensemble_workspace_bytes(self.handle, byref(nbytes)))
        self.work = torch.empty(nbytes.value, dtype=torch.uint8, device=self.device)
        self._captured = None

    @property
    def members(self) -> int:
        return sum(self.batches)

    def _ptrs(self, states):
        if len(states) != len(self.models):
            raise ValueError("need one state tensor per group")
        for k, (s, m, b) in enumerate(zip(states, self.models, self.batches)):
            L = m.sh.l_max
            if (tuple(s.shape) != (b, L + 1, L + 1) or s.dtype != torch.complex128 or not s.is_cuda
                    or not s.is_contiguous()):
                raise ValueError(f"group {k}: expected a contiguous complex128 CUDA tensor [{b}, {L + 1}, {L + 1}]")
        return (c_void_p * len(states))(*[s.data_ptr() for s in states])

    def rk4(self, states, dt: float, nsteps: int = 1):
        """nsteps RK4 steps of every group, in place."""
        p = self._ptrs(states)
        check(_lib.load().aeolus_ensemble_bve_rk4(self.handle, ctypes.cast(p, ctypes.POINTER(c_void_p)), float(dt),
                                                  int(nsteps), c_void_p(self.work.data_ptr()), self.work.numel(),
                                                  _stream(self.device)))
        return states

    def capture(self, states, dt: float, stream: torch.cuda.Stream | None = None):
        """Capture one RK4 step of these (fixed) state tensors into a CUDA
        graph on a side stream; replay with :meth:`replay`."""
        p = self._ptrs(states)
        s = stream or torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        check(_lib.load().aeolus_ensemble_capture(self.handle, ctypes.cast(p, ctypes.POINTER(c_void_p)), float(dt),
                                                  c_void_p(self.work.data_ptr()), self.work.numel(),
                                                  c_void_p(s.cuda_stream)))
        torch.cuda.current_stream(self.device).wait_stream(s)
        self._captured = (list(states), s)

    def replay(self, nsteps: int = 1):
        if self._captured is None:
            raise RuntimeError("no captured step: call capture() first")
        s = torch.cuda.current_stream(self.device)
        check(_lib.load().aeolus_ensemble_launch(self.handle, int(nsteps), c_void_p(s.cuda_stream)))

    def autotune(self, states) -> str:
        """Pick launch shapes per group by timing candidates; returns the report."""
        p = self._ptrs(states)
        buf = ctypes.create_string_buffer(1 << 14)
        check(_lib.load().aeolus_ensemble_autotune(self.handle, ctypes.cast(p, ctypes.POINTER(c_void_p)),
                                                   c_void_p(self.work.data_ptr()), self.work.numel(),
                                                   _stream(self.device), buf, len(buf)))
        self._captured = None
        return buf.value.decode()

    def close(self):
        if self.handle:
            _lib.load().aeolus_ensemble_destroy(self.handle)
            self.handle = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
