"""Batched uneven ensembles: members of different l_max advanced together.

Each group is a model (:class:`~aeolus_gb300.barotropic.BarotropicVorticity`
or :class:`~aeolus_gb300.shallow_water.ShallowWaterModel`, each with its own
Gauss grid and product-space plan) with a batch of members; every RK4 stage
launches each stage kernel once for all groups (``aeolus_ensemble_bve_rk4``,
``aeolus_ensemble_swe_rk4``), a whole step can be captured into a CUDA graph
and replayed (``aeolus_ensemble_capture`` / ``aeolus_ensemble_launch``), and
``autotune`` times candidate launch shapes per group on the ensemble's own
states (``aeolus_ensemble_autotune``).

The reference runs one state per process (run/bve/runner.py:211-216,
run/engine.py:406-431); the per-member arithmetic here is that of the
models' own ``rk4``.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_int, c_size_t, c_void_p

import torch

from . import _lib
from ._lib import check
from .ops import _stream


class _Ensemble:
    """Shared workspace, graph capture / replay and autotuning."""

    _fields = 1  # state fields per member

    def _finish_init(self):
        nbytes = c_size_t()
        check(_lib.load().aeolus_ensemble_workspace_bytes(self.handle, byref(nbytes)))
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
            shape = (b, L + 1, L + 1) if self._fields == 1 else (b, self._fields, L + 1, L + 1)
            if tuple(s.shape) != shape or s.dtype != torch.complex128 or not s.is_cuda or not s.is_contiguous():
                raise ValueError(f"group {k}: expected a contiguous complex128 CUDA tensor {list(shape)}")
        return (c_void_p * len(states))(*[s.data_ptr() for s in states])

    def _step(self, fn, states, dt: float, nsteps: int):
        p = self._ptrs(states)
        check(fn(self.handle, ctypes.cast(p, ctypes.POINTER(c_void_p)), float(dt), int(nsteps),
                 c_void_p(self.work.data_ptr()), self.work.numel(), _stream(self.device)))
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
        if getattr(self, "handle", None):
            _lib.load().aeolus_ensemble_destroy(self.handle)
            self.handle = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check_groups(models, batches):
    if len(models) != len(batches) or not models:
        raise ValueError("need one batch size per model")
    return list(models), [int(b) for b in batches]


class BarotropicEnsemble(_Ensemble):
    """BVE groups; states [batch, L+1, L+1] per group."""

    _fields = 1

    def __init__(self, models, batches):
        self.models, self.batches = _check_groups(models, batches)
        self.device = self.models[0].f_lm.device
        n = len(self.models)
        plans = (c_void_p * n)(*[m._plan.handle.value for m in self.models])
        bs = (c_int * n)(*self.batches)
        prm = (_lib.BveParams * n)(*[_lib.BveParams(m.R, m.Omega, m.nu) for m in self.models])
        self.handle = c_void_p()
        check(_lib.load().aeolus_ensemble_create(n, ctypes.cast(plans, ctypes.POINTER(c_void_p)), bs, prm,
                                                 byref(self.handle)))
        self._finish_init()

    def rk4(self, states, dt: float, nsteps: int = 1):
        """nsteps RK4 steps of every group, in place."""
        return self._step(_lib.load().aeolus_ensemble_bve_rk4, states, dt, nsteps)


class ShallowWaterEnsemble(_Ensemble):
    """SWE groups; states [batch, 3, L+1, L+1] per group (no in-step state
    checks: the members' status bits are those of the single-model rk4)."""

    _fields = 3

    def __init__(self, models, batches):
        self.models, self.batches = _check_groups(models, batches)
        self.device = self.models[0]._plan.device
        n = len(self.models)
        plans = (c_void_p * n)(*[m._plan.handle.value for m in self.models])
        bs = (c_int * n)(*self.batches)
        # each model keeps its forcing tensor (bottom topography) alive for the ensemble's lifetime
        prm = (_lib.SweParams * n)(*[_lib.SweParams(m.R, m.Omega, m.gravity, m.mean_depth, m.nu4, m.forcing_ptr())
                                     for m in self.models])
        self.handle = c_void_p()
        check(_lib.load().aeolus_ensemble_create_swe(n, ctypes.cast(plans, ctypes.POINTER(c_void_p)), bs, prm,
                                                     byref(self.handle)))
        self._finish_init()

    def rk4(self, states, dt: float, nsteps: int = 1):
        """nsteps RK4 steps of every group, in place."""
        return self._step(_lib.load().aeolus_ensemble_swe_rk4, states, dt, nsteps)
