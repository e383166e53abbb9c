"""PyTorch custom ops over the C ABI (device tensors in, device tensors out).

Every op runs on torch's current CUDA stream, allocates its scratch from
torch's caching allocator and calls exactly one entry point of
``libaeolus_gb300.so``.  Spectral tensors are complex128 ``[..., L+1, L+1]``
(the reference layout), grid tensors float64 ``[..., n_points]``.
"""
from __future__ import annotations

import ctypes
import math
import threading
from ctypes import byref, c_double, c_int, c_long, c_size_t, c_void_p

import numpy as np
import torch

from . import _lib
from ._lib import TUNING_KNOBS, check

_PLANS: dict[int, "Plan"] = {}
_LOCK = threading.Lock()


def _ptr(t: torch.Tensor | None) -> c_void_p:
    return c_void_p(0 if t is None else t.data_ptr())


def _stream(device: torch.device) -> c_void_p:
    return c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _require_cuda(t: torch.Tensor, name: str):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the GB300 path has no CPU fallback)")


class Plan:
    """Owner of one C plan handle (Gauss grid or point set)."""

    def __init__(self, handle: int, device: torch.device):
        self.handle = c_void_p(handle)
        self.device = device
        lib = _lib.load()
        kind, nlat, nlon, lmax, npts = c_int(), c_int(), c_int(), c_int(), c_long()
        check(lib.aeolus_plan_info(self.handle, byref(kind), byref(nlat), byref(nlon), byref(lmax), byref(npts)))
        self.kind, self.nlat, self.nlon = kind.value, nlat.value, nlon.value
        self.lmax, self.n_points = lmax.value, npts.value
        self.precision = _lib.PREC_FP64
        self.id = handle
        with _LOCK:
            _PLANS[self.id] = self

    @classmethod
    def gauss(cls, nlat: int, nlon: int, lmax: int, radius: float = 1.0, device=None) -> "Plan":
        device = torch.device(device or "cuda")
        lib = _lib.load()
        h = c_void_p()
        with torch.cuda.device(device):
            check(lib.aeolus_plan_create_gauss(int(nlat), int(nlon), int(lmax), float(radius), 0, byref(h)))
        return cls(h.value, device)

    @classmethod
    def points(cls, lat, lon, weights, lmax: int, radius: float = 1.0, device=None) -> "Plan":
        device = torch.device(device or "cuda")
        lat = np.ascontiguousarray(lat, dtype=np.float64)
        lon = np.ascontiguousarray(lon, dtype=np.float64)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        if lat.shape != lon.shape or lat.ndim != 1:
            raise ValueError("Latitude and Longitude arrays must have the same 1-D shape.")
        lib = _lib.load()
        h = c_void_p()
        with torch.cuda.device(device):
            check(lib.aeolus_plan_create_points(lat.size, lat.ctypes.data_as(c_void_p), lon.ctypes.data_as(c_void_p),
                                                None if w is None else w.ctypes.data_as(c_void_p), int(lmax),
                                                float(radius), 0, byref(h)))
        return cls(h.value, device)

    def nodes(self):
        lat = np.empty(self.nlat)
        w = np.empty(self.nlat)
        check(_lib.load().aeolus_plan_nodes(self.handle, lat.ctypes.data_as(c_void_p), w.ctypes.data_as(c_void_p)))
        return lat, w

    def set_precision(self, precision: int, slices: int = 0):
        check(_lib.load().aeolus_plan_set_precision(self.handle, int(precision), int(slices)))
        self.precision = int(precision)

    def tuning(self) -> tuple[int, int, int, int, int]:
        """(bc_synth, bc_anal, row_threads, synth_slice_members,
        anal_slice_members); 0 = heuristic."""
        k = (c_int * TUNING_KNOBS)()
        check(_lib.load().aeolus_plan_get_tuning(self.handle, k))
        return tuple(k)

    def set_tuning(self, knobs) -> None:
        if len(knobs) != TUNING_KNOBS:
            raise ValueError(f"set_tuning takes {TUNING_KNOBS} knobs")
        k = (c_int * TUNING_KNOBS)(*[int(x) for x in knobs])
        check(_lib.load().aeolus_plan_set_tuning(self.handle, k))

    def workspace(self, op: int, batch: int) -> torch.Tensor:
        n = c_size_t()
        check(_lib.load().aeolus_workspace_bytes(self.handle, int(op), int(batch), byref(n)))
        return torch.empty(n.value, dtype=torch.uint8, device=self.device)

    def close(self):
        if self.handle:
            with _LOCK:
                _PLANS.pop(self.id, None)
            _lib.load().aeolus_plan_destroy(self.handle)
            self.handle = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def geodesic_build(resolution: int, radius: float = 1.0, device=None) -> dict:
    """Icosahedral geodesic point set built on the device by
    ``aeolus_geodesic_build`` (geodesic_grid.py:31-266): points, faces,
    lat/lon, barycentric cell areas and the minimum edge length."""
    device = torch.device(device or "cuda")
    lib = _lib.load()
    nv, nf, nb = c_long(), c_long(), c_size_t()
    check(lib.aeolus_geodesic_sizes(int(resolution), byref(nv), byref(nf), byref(nb)))
    f64 = dict(dtype=torch.float64, device=device)
    with torch.cuda.device(device):
        pts = torch.empty((nv.value, 3), **f64)
        faces = torch.empty((nf.value, 3), dtype=torch.int32, device=device)
        lat, lon, areas = (torch.empty(nv.value, **f64) for _ in range(3))
        min_edge = torch.empty(1, **f64)
        status = torch.zeros(1, dtype=torch.int32, device=device)
        work = torch.empty(max(nb.value, 1), dtype=torch.uint8, device=device)
        check(lib.aeolus_geodesic_build(int(resolution), float(radius), _ptr(pts), _ptr(faces), _ptr(lat), _ptr(lon),
                                        _ptr(areas), _ptr(min_edge), _ptr(status), _ptr(work), nb.value,
                                        _stream(device)))
    if int(status.item()) != 0:
        raise RuntimeError("geodesic build: a vertex has more than 6 incident faces")
    return {"points": pts, "faces": faces, "lat": lat, "lon": lon, "areas": areas,
            "min_edge": float(min_edge.item())}


def _spec_shape(L: int):
    return (L + 1, L + 1)


def _flat_spec(t: torch.Tensor, L: int, nf: int = 1) -> tuple[torch.Tensor, tuple]:
    _require_cuda(t, "coefficients")
    tail = (nf, L + 1, L + 1) if nf > 1 else (L + 1, L + 1)
    if tuple(t.shape[-len(tail):]) != tail:
        raise ValueError(f"expected coefficients shaped [..., {', '.join(map(str, tail))}], got {tuple(t.shape)}")
    lead = tuple(t.shape[:-len(tail)])
    return t.to(torch.complex128).contiguous().reshape((-1,) + tail), lead


# ------------------------------------------------------------------ ops
@torch.library.custom_op("aeolus::synthesize", mutates_args=())
def synthesize(plan_id: int, coeffs: torch.Tensor) -> torch.Tensor:
    """Batched synthesis, fast_geodesic_sh.py:89-107."""
    p = _PLANS[plan_id]
    c, lead = _flat_spec(coeffs, p.lmax)
    B = c.shape[0]
    out = torch.empty((B, p.n_points), dtype=torch.float64, device=c.device)
    if B:
        w = p.workspace(_lib.OP_SYNTHESIZE, B)
        check(_lib.load().aeolus_synthesize(p.handle, _ptr(c), _ptr(out), B, _ptr(w), w.numel(), _stream(c.device)))
    return out.reshape(lead + (p.n_points,))


@torch.library.custom_op("aeolus::analyze", mutates_args=())
def analyze(plan_id: int, grid: torch.Tensor) -> torch.Tensor:
    """Batched analysis, fast_geodesic_sh.py:68-87."""
    p = _PLANS[plan_id]
    _require_cuda(grid, "grid values")
    if grid.shape[-1] != p.n_points:
        raise ValueError(f"expected [..., {p.n_points}] grid values, got {tuple(grid.shape)}")
    lead = tuple(grid.shape[:-1])
    g = grid.to(torch.float64).contiguous().reshape(-1, p.n_points)
    B = g.shape[0]
    out = torch.empty((B,) + _spec_shape(p.lmax), dtype=torch.complex128, device=g.device)
    if B:
        w = p.workspace(_lib.OP_ANALYZE, B)
        check(_lib.load().aeolus_analyze(p.handle, _ptr(g), _ptr(out), B, _ptr(w), w.numel(), _stream(g.device)))
    return out.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::vector_curl_div", mutates_args=())
def vector_curl_div(plan_id: int, radius: float, f_east: torch.Tensor, f_north: torch.Tensor,
                    truncate: bool) -> torch.Tensor:
    """[2, ..., L+1, L+1] (curl, div) of tangent fields on the plan's points by
    the weak form, spectral_operators.py:399-492; the plan is the one-degree-
    extended analysis plan (l_max = L + 1) on the product points."""
    p = _PLANS[plan_id]
    _require_cuda(f_east, "eastward component")
    _require_cuda(f_north, "northward component")
    if f_east.shape != f_north.shape or f_east.shape[-1] != p.n_points:
        raise ValueError(f"expected two [..., {p.n_points}] components, got {tuple(f_east.shape)} and "
                         f"{tuple(f_north.shape)}")
    lead = tuple(f_east.shape[:-1])
    fe = torch.stack((f_east.to(torch.float64).reshape(-1, p.n_points),
                      f_north.to(torch.float64).reshape(-1, p.n_points)), dim=1).contiguous()
    B, L = fe.shape[0], p.lmax - 1
    out = torch.empty((2, B, L + 1, L + 1), dtype=torch.complex128, device=fe.device)
    if B:
        w = p.workspace(_lib.OP_VECTOR_CURL_DIV, B)
        check(_lib.load().aeolus_vector_curl_div(p.handle, float(radius), _ptr(fe), _ptr(out[0]), _ptr(out[1]), B,
                                                 1 if truncate else 0, _ptr(w), w.numel(), _stream(fe.device)))
    return out.reshape((2,) + lead + (L + 1, L + 1))


@torch.library.custom_op("aeolus::spectral_op", mutates_args=())
def spectral_op(op: int, radius: float, coeffs: torch.Tensor) -> torch.Tensor:
    """Diagonal / tridiagonal spectral operator (aeolus_spectral_op ids)."""
    L = coeffs.shape[-1] - 1
    c, lead = _flat_spec(coeffs, L)
    out = torch.empty_like(c)
    if c.shape[0]:
        check(_lib.load().aeolus_spectral_op(int(op), L, float(radius), _ptr(c), _ptr(out), c.shape[0],
                                             _stream(c.device)))
    return out.reshape(lead + _spec_shape(L))


@torch.library.custom_op("aeolus::jacobian", mutates_args=())
def jacobian(plan_id: int, a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    p = _PLANS[plan_id]
    ca, lead = _flat_spec(a, p.lmax)
    cb, _ = _flat_spec(b, p.lmax)
    out = torch.empty_like(ca)
    B = ca.shape[0]
    if B:
        w = p.workspace(_lib.OP_JACOBIAN, B)
        check(_lib.load().aeolus_jacobian(p.handle, _ptr(ca), _ptr(cb), _ptr(out), B, _ptr(w), w.numel(),
                                          _stream(ca.device)))
    return out.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::winds", mutates_args=())
def winds(plan_id: int, radius: float, psi: torch.Tensor, chi: torch.Tensor | None) -> torch.Tensor:
    """[2, ..., n_points] (u, v)."""
    p = _PLANS[plan_id]
    cp_, lead = _flat_spec(psi, p.lmax)
    cc = _flat_spec(chi, p.lmax)[0] if chi is not None else None
    B = cp_.shape[0]
    out = torch.empty((2, B, p.n_points), dtype=torch.float64, device=cp_.device)
    if B:
        w = p.workspace(_lib.OP_WINDS, B)
        check(_lib.load().aeolus_winds(p.handle, float(radius), _ptr(cp_), _ptr(cc), _ptr(out), B, _ptr(w),
                                       w.numel(), _stream(cp_.device)))
    return out.reshape((2,) + lead + (p.n_points,))


def _bve_params(radius, omega, nu):
    return _lib.BveParams(float(radius), float(omega), float(nu))


def _swe_params(radius, omega, gravity, mean_depth, nu4, forcing=None, L=None, device=None):
    """The C parameter block; `forcing` is the constant [3, L+1, L+1] complex
    spectral forcing of bottom topography (or None)."""
    fp = None
    if forcing is not None:
        if forcing.dtype != torch.complex128 or tuple(forcing.shape) != (3, L + 1, L + 1) \
                or not forcing.is_contiguous() or forcing.device != device:
            raise ValueError(f"forcing must be a contiguous complex128 [3, {L + 1}, {L + 1}] tensor on {device}")
        fp = forcing.data_ptr()
    return _lib.SweParams(float(radius), float(omega), float(gravity), float(mean_depth), float(nu4), fp)


@torch.library.custom_op("aeolus::bve_tendency", mutates_args=())
def bve_tendency(plan_id: int, radius: float, omega: float, nu: float, zeta: torch.Tensor,
                 forcing: torch.Tensor | None) -> torch.Tensor:
    p = _PLANS[plan_id]
    z, lead = _flat_spec(zeta, p.lmax)
    f = _flat_spec(forcing, p.lmax)[0] if forcing is not None else None
    out = torch.empty_like(z)
    B = z.shape[0]
    if B:
        w = p.workspace(_lib.OP_BVE_TENDENCY, B)
        prm = _bve_params(radius, omega, nu)
        check(_lib.load().aeolus_bve_tendency(p.handle, byref(prm), _ptr(z), _ptr(f), _ptr(out), B, _ptr(w),
                                              w.numel(), _stream(z.device)))
    return out.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::swe_tendency", mutates_args=())
def swe_tendency(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float, nu4: float,
                 state: torch.Tensor, forcing: torch.Tensor | None = None) -> torch.Tensor:
    p = _PLANS[plan_id]
    s, lead = _flat_spec(state, p.lmax, 3)
    out = torch.empty_like(s)
    B = s.shape[0]
    if B:
        w = p.workspace(_lib.OP_SWE_TENDENCY, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, nu4, forcing, p.lmax, s.device)
        check(_lib.load().aeolus_swe_tendency(p.handle, byref(prm), _ptr(s), _ptr(out), B, _ptr(w), w.numel(),
                                              _stream(s.device)))
    return out.reshape(lead + (3,) + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::bve_rk4", mutates_args=())
def bve_rk4(plan_id: int, radius: float, omega: float, nu: float, zeta: torch.Tensor, dt: float,
            nsteps: int) -> torch.Tensor:
    p = _PLANS[plan_id]
    z, lead = _flat_spec(zeta, p.lmax)
    y = z.clone()
    B = y.shape[0]
    if B and nsteps > 0:
        w = p.workspace(_lib.OP_BVE_RK4, B)
        prm = _bve_params(radius, omega, nu)
        check(_lib.load().aeolus_bve_rk4(p.handle, byref(prm), _ptr(y), B, float(dt), int(nsteps), _ptr(w),
                                         w.numel(), _stream(y.device)))
    return y.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::swe_rk4", mutates_args=())
def swe_rk4(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float, nu4: float,
            state: torch.Tensor, dt: float, nsteps: int,
            forcing: torch.Tensor | None = None) -> tuple[torch.Tensor, torch.Tensor]:
    """(new state, per-member status bits OR-ed over every stage)."""
    p = _PLANS[plan_id]
    s, lead = _flat_spec(state, p.lmax, 3)
    y = s.clone()
    B = y.shape[0]
    status = torch.zeros(B, dtype=torch.int32, device=y.device)
    if B and nsteps > 0:
        w = p.workspace(_lib.OP_SWE_RK4, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, nu4, forcing, p.lmax, y.device)
        check(_lib.load().aeolus_swe_rk4(p.handle, byref(prm), _ptr(y), B, float(dt), int(nsteps), _ptr(status),
                                         _ptr(w), w.numel(), _stream(y.device)))
    return y.reshape(lead + (3,) + _spec_shape(p.lmax)), status.reshape(lead)


def swe_rk4_inplace(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float, nu4: float,
                    state: torch.Tensor, dt: float, nsteps: int, forcing: torch.Tensor | None = None) -> torch.Tensor:
    """swe_rk4 on a contiguous [B, 3, L+1, L+1] device state in place (no
    copy of the input); returns the per-member status bits."""
    p = _PLANS[plan_id]
    if not state.is_contiguous():
        raise ValueError("swe_rk4_inplace needs a contiguous state")
    B = state.shape[0]
    status = torch.zeros(B, dtype=torch.int32, device=state.device)
    if B and nsteps > 0:
        w = p.workspace(_lib.OP_SWE_RK4, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, nu4, forcing, p.lmax, state.device)
        check(_lib.load().aeolus_swe_rk4(p.handle, byref(prm), _ptr(state), B, float(dt), int(nsteps),
                                         _ptr(status), _ptr(w), w.numel(), _stream(state.device)))
    return status


@torch.library.custom_op("aeolus::swe_validate", mutates_args=())
def swe_validate(state_plan: int, product_plan: int, radius: float, omega: float, gravity: float,
                 mean_depth: float, state: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """(status bits [B], extrema [B, 2] of Phi0 + phi over both samplings)."""
    p = _PLANS[state_plan]
    q = _PLANS[product_plan]
    s, lead = _flat_spec(state, p.lmax, 3)
    B = s.shape[0]
    status = torch.zeros(B, dtype=torch.int32, device=s.device)
    ext = torch.empty((B, 2), dtype=torch.float64, device=s.device)
    if B:
        n = max(p.workspace(_lib.OP_SWE_VALIDATE, B).numel(), q.workspace(_lib.OP_SWE_VALIDATE, B).numel())
        w = torch.empty(n, dtype=torch.uint8, device=s.device)
        prm = _swe_params(radius, omega, gravity, mean_depth, 0.0)
        check(_lib.load().aeolus_swe_validate(p.handle, q.handle, byref(prm), _ptr(s), _ptr(status), _ptr(ext), B,
                                              _ptr(w), w.numel(), _stream(s.device)))
    return status.reshape(lead), ext.reshape(lead + (2,))


@torch.library.custom_op("aeolus::bve_spectral_diagnostics", mutates_args=())
def bve_spectral_diagnostics(radius: float, omega: float, zeta: torch.Tensor) -> torch.Tensor:
    L = zeta.shape[-1] - 1
    z, lead = _flat_spec(zeta, L)
    out = torch.empty((z.shape[0], 6), dtype=torch.float64, device=z.device)
    if z.shape[0]:
        check(_lib.load().aeolus_bve_spectral_diagnostics(L, float(radius), float(omega), _ptr(z), _ptr(out),
                                                          z.shape[0], _stream(z.device)))
    return out.reshape(lead + (6,))


@torch.library.custom_op("aeolus::swe_invariants", mutates_args=())
def swe_invariants(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float,
                   state: torch.Tensor) -> torch.Tensor:
    p = _PLANS[plan_id]
    s, lead = _flat_spec(state, p.lmax, 3)
    B = s.shape[0]
    out = torch.empty((B, 5), dtype=torch.float64, device=s.device)
    if B:
        w = p.workspace(_lib.OP_SWE_INVARIANTS, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, 0.0)
        check(_lib.load().aeolus_swe_invariants(p.handle, byref(prm), _ptr(s), _ptr(out), B, _ptr(w), w.numel(),
                                                _stream(s.device)))
    return out.reshape(lead + (5,))


# ------------------------------------------------------------ adjoints
@torch.library.custom_op("aeolus::synthesize_adjoint", mutates_args=())
def synthesize_adjoint(plan_id: int, grid_bar: torch.Tensor) -> torch.Tensor:
    """S^T grid_bar (the backward of synthesize)."""
    p = _PLANS[plan_id]
    _require_cuda(grid_bar, "grid adjoint")
    if grid_bar.shape[-1] != p.n_points:
        raise ValueError(f"expected [..., {p.n_points}] grid values, got {tuple(grid_bar.shape)}")
    lead = tuple(grid_bar.shape[:-1])
    g = grid_bar.to(torch.float64).contiguous().reshape(-1, p.n_points)
    B = g.shape[0]
    out = torch.empty((B,) + _spec_shape(p.lmax), dtype=torch.complex128, device=g.device)
    if B:
        w = p.workspace(_lib.OP_SYNTHESIZE_ADJOINT, B)
        check(_lib.load().aeolus_synthesize_adjoint(p.handle, _ptr(g), _ptr(out), B, _ptr(w), w.numel(),
                                                    _stream(g.device)))
    return out.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::analyze_adjoint", mutates_args=())
def analyze_adjoint(plan_id: int, coeffs_bar: torch.Tensor) -> torch.Tensor:
    """A^T coeffs_bar (the backward of analyze)."""
    p = _PLANS[plan_id]
    c, lead = _flat_spec(coeffs_bar, p.lmax)
    B = c.shape[0]
    out = torch.empty((B, p.n_points), dtype=torch.float64, device=c.device)
    if B:
        w = p.workspace(_lib.OP_ANALYZE_ADJOINT, B)
        check(_lib.load().aeolus_analyze_adjoint(p.handle, _ptr(c), _ptr(out), B, _ptr(w), w.numel(),
                                                 _stream(c.device)))
    return out.reshape(lead + (p.n_points,))


@torch.library.custom_op("aeolus::swe_tendency_adjoint", mutates_args=())
def swe_tendency_adjoint(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float, nu4: float,
                         state: torch.Tensor, tend_bar: torch.Tensor) -> torch.Tensor:
    """(d tendency / d state)^T tend_bar."""
    p = _PLANS[plan_id]
    s, lead = _flat_spec(state, p.lmax, 3)
    kb, _ = _flat_spec(tend_bar, p.lmax, 3)
    out = torch.empty_like(s)
    B = s.shape[0]
    if B:
        w = p.workspace(_lib.OP_SWE_TENDENCY_ADJOINT, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, nu4)
        check(_lib.load().aeolus_swe_tendency_adjoint(p.handle, byref(prm), _ptr(s), _ptr(kb), _ptr(out), B,
                                                      _ptr(w), w.numel(), _stream(s.device)))
    return out.reshape(lead + (3,) + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::bve_tendency_adjoint", mutates_args=())
def bve_tendency_adjoint(plan_id: int, radius: float, omega: float, nu: float, zeta: torch.Tensor,
                         tend_bar: torch.Tensor) -> torch.Tensor:
    p = _PLANS[plan_id]
    z, lead = _flat_spec(zeta, p.lmax)
    kb, _ = _flat_spec(tend_bar, p.lmax)
    out = torch.empty_like(z)
    B = z.shape[0]
    if B:
        w = p.workspace(_lib.OP_BVE_TENDENCY_ADJOINT, B)
        prm = _bve_params(radius, omega, nu)
        check(_lib.load().aeolus_bve_tendency_adjoint(p.handle, byref(prm), _ptr(z), _ptr(kb), _ptr(out), B,
                                                      _ptr(w), w.numel(), _stream(z.device)))
    return out.reshape(lead + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::swe_rk4_adjoint", mutates_args=())
def swe_rk4_adjoint(plan_id: int, radius: float, omega: float, gravity: float, mean_depth: float, nu4: float,
                    state: torch.Tensor, state_bar: torch.Tensor, dt: float,
                    forcing: torch.Tensor | None = None) -> torch.Tensor:
    """Adjoint of one RK4 step taken from `state`: maps the adjoint of the
    step's output to that of its input (a constant forcing only shifts the
    recomputed stage inputs)."""
    p = _PLANS[plan_id]
    s, lead = _flat_spec(state, p.lmax, 3)
    yb = _flat_spec(state_bar, p.lmax, 3)[0].clone()
    B = s.shape[0]
    if B:
        w = p.workspace(_lib.OP_SWE_RK4_ADJOINT, B)
        prm = _swe_params(radius, omega, gravity, mean_depth, nu4, forcing, p.lmax, s.device)
        check(_lib.load().aeolus_swe_rk4_adjoint(p.handle, byref(prm), _ptr(s), _ptr(yb), B, float(dt), _ptr(w),
                                                 w.numel(), _stream(s.device)))
    return yb.reshape(lead + (3,) + _spec_shape(p.lmax))


@torch.library.custom_op("aeolus::bve_rk4_adjoint", mutates_args=())
def bve_rk4_adjoint(plan_id: int, radius: float, omega: float, nu: float, zeta: torch.Tensor,
                    zeta_bar: torch.Tensor, dt: float) -> torch.Tensor:
    p = _PLANS[plan_id]
    z, lead = _flat_spec(zeta, p.lmax)
    yb = _flat_spec(zeta_bar, p.lmax)[0].clone()
    B = z.shape[0]
    if B:
        w = p.workspace(_lib.OP_BVE_RK4_ADJOINT, B)
        prm = _bve_params(radius, omega, nu)
        check(_lib.load().aeolus_bve_rk4_adjoint(p.handle, byref(prm), _ptr(z), _ptr(yb), B, float(dt), _ptr(w),
                                                 w.numel(), _stream(z.device)))
    return yb.reshape(lead + _spec_shape(p.lmax))


# Autograd: the backward of each transform is its hand-written transpose.
def _synth_setup(ctx, inputs, output):
    ctx.plan_id = inputs[0]


def _synth_backward(ctx, grad):
    return None, synthesize_adjoint(ctx.plan_id, grad.contiguous())


def _anal_backward(ctx, grad):
    return None, analyze_adjoint(ctx.plan_id, grad.contiguous())


def _synth_adj_backward(ctx, grad):
    return None, synthesize(ctx.plan_id, grad.contiguous())


def _anal_adj_backward(ctx, grad):
    return None, analyze(ctx.plan_id, grad.contiguous())


torch.library.register_autograd("aeolus::synthesize", _synth_backward, setup_context=_synth_setup)
torch.library.register_autograd("aeolus::analyze", _anal_backward, setup_context=_synth_setup)
torch.library.register_autograd("aeolus::synthesize_adjoint", _synth_adj_backward, setup_context=_synth_setup)
torch.library.register_autograd("aeolus::analyze_adjoint", _anal_adj_backward, setup_context=_synth_setup)


def f10(omega: float) -> float:
    """Spectral (1,0) coefficient of f = 2 Omega sin(lat), barotropic.py:59-61."""
    return 2.0 * omega * math.sqrt(4.0 * math.pi / 3.0)


def rk4_stage(stage: int, dt: float, y0: torch.Tensor, k: torch.Tensor, ystage: torch.Tensor,
              acc: torch.Tensor) -> None:
    """In place: one RK4 stage update on the device (aeolus_rk4_stage), the
    reference's rk4_step_array order of operations (run/engine.py:406-431);
    complex128 CUDA tensors of one shape, contiguous."""
    for name, t in (("y0", y0), ("k", k), ("ystage", ystage), ("acc", acc)):
        _require_cuda(t, name)
        if t.dtype != torch.complex128 or not t.is_contiguous() or t.shape != y0.shape:
            raise ValueError(f"rk4_stage: {name} must be a contiguous complex128 tensor shaped like y0")
    check(_lib.load().aeolus_rk4_stage(int(stage), float(dt), _ptr(y0), _ptr(k), _ptr(ystage), _ptr(acc),
                                       y0.numel(), _stream(y0.device)))
