"""Rotating shallow-water core on the GB300 path.

Mirrors src/planetary_sandbox/physics/shallow_water.py:102-539, bottom
topography included (constant spectral forcing terms).  ``tendency`` is one
fused chain on the product space: nine
syntheses (u cos, v cos, eta_lam, eta_snt, phi_lam, phi_snt, zeta, delta,
phi), the pointwise flux products, four analyses, the 2/3 cut and the exact
linear terms.  ``rk4`` advances whole steps on the device and checks every
stage state (NaN/Inf, fluid thickness) without host synchronisation.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from . import _lib
from .ops import spectral_op, swe_invariants, swe_rk4, swe_rk4_inplace, swe_tendency, swe_validate, winds

WILLIAMSON_GRAVITY = 9.80616
ZETA, DELTA, PHI = 0, 1, 2
PROGNOSTICS = ("zeta", "delta", "phi")


def _or_bits(status: torch.Tensor) -> int:
    bits = 0
    for v in status.reshape(-1).tolist():
        bits |= int(v)
    return bits


class ShallowWaterStateError(ValueError):
    """A shallow-water state violated a hard physical/numerical constraint."""


@dataclass
class ShallowWaterState:
    coeffs: torch.Tensor

    @classmethod
    def from_fields(cls, zeta_lm, delta_lm, phi_lm) -> "ShallowWaterState":
        return cls(torch.stack([torch.as_tensor(x, dtype=torch.complex128) for x in (zeta_lm, delta_lm, phi_lm)]))

    @classmethod
    def zeros(cls, l_max: int, device=None) -> "ShallowWaterState":
        n = l_max + 1
        return cls(torch.zeros((3, n, n), dtype=torch.complex128, device=device or "cuda"))

    zeta = property(lambda self: self.coeffs[ZETA])
    delta = property(lambda self: self.coeffs[DELTA])
    phi = property(lambda self: self.coeffs[PHI])


class ShallowWaterModel:
    _MONOPOLE_RTOL = 1e-10

    def __init__(self, planet, *, gravity: float = WILLIAMSON_GRAVITY, mean_depth: float,
                 hyperdiffusion_nu4: float = 0.0, topography=None):
        if not (math.isfinite(gravity) and gravity > 0):
            raise ValueError(f"gravity must be finite and > 0, got {gravity}")
        if not (math.isfinite(mean_depth) and mean_depth > 0):
            raise ValueError(f"mean_depth must be finite and > 0, got {mean_depth}")
        if not (math.isfinite(hyperdiffusion_nu4) and hyperdiffusion_nu4 >= 0):
            raise ValueError(f"hyperdiffusion_nu4 must be finite and >= 0, got {hyperdiffusion_nu4}")
        self.planet = planet
        self.sh = planet.sh
        self.so = planet.so
        self.grid = planet.grid
        self.R = float(planet.params.radius)
        self.Omega = float(planet.params.angular_velocity)
        self.gravity = float(gravity)
        self.mean_depth = float(mean_depth)
        self.phi0 = self.gravity * self.mean_depth
        self.nu4 = float(hyperdiffusion_nu4)
        self.l_max = self.sh.l_max
        dev = self.sh.weights.device
        self.f_lm = torch.zeros((self.l_max + 1, self.l_max + 1), dtype=torch.complex128, device=dev)
        self.f_lm[1, 0] = 2.0 * self.Omega * math.sqrt(4.0 * math.pi / 3.0)
        l = torch.arange(self.l_max + 1, dtype=torch.float64, device=dev)
        self.lap_eigs = -l * (l + 1.0) / self.R ** 2
        self._ps = self.so.backend.product_space(self.so.product_quadrature)
        self._plan = self._ps.sh.plan
        self._state_plan = self.sh.plan
        self._set_topography(topography)

    # -- bottom topography (shallow_water.py:226-271) ------------------------
    def _set_topography(self, topography):
        """phi_s = g h_s enters as constant spectral terms: -lap(phi_s) in the
        divergence tendency and, with hyperdiffusion, -nu4 lap^2 phi_s' (the
        mean-removed anomaly) in the geopotential tendency.  They are handed
        to the kernels as one [3, L+1, L+1] forcing array; a flat bottom
        passes none, so its path is unchanged."""
        from .topography import Topography

        n = self.l_max + 1
        dev = self.lap_eigs.device
        if topography is None:
            topography = Topography.flat(self.l_max)
        if topography.l_max != self.l_max:
            raise ValueError(f"topography truncation l_max={topography.l_max} does not match the model's "
                             f"l_max={self.l_max}")
        self.topography = topography
        self.has_topography = not topography.is_flat
        self.forcing = None
        if self.has_topography:
            self.phi_s_lm = topography.surface_geopotential_lm(self.gravity).to(dev)
            self.phi_s_anom_lm = self.phi_s_lm.clone()
            self.phi_s_anom_lm[0, 0] = 0.0
            lap = self.lap_eigs[:, None]
            f = torch.zeros((3, n, n), dtype=torch.complex128, device=dev)
            f[DELTA] = -(lap * self.phi_s_lm)
            if self.nu4 > 0.0:
                f[PHI] = -(self.nu4 * lap ** 2 * self.phi_s_anom_lm)
            f[:, 0, :] = 0.0
            self.forcing = f.contiguous()
            samplings = [self.sh] + ([self._ps.sh] if self._ps.sh is not self.sh else [])
            ext = [torch.aminmax(topography.elevation_on(sh)) for sh in samplings]
            self.surface_elevation_extrema = (min(float(e.min) for e in ext), max(float(e.max) for e in ext))
            self._phi_s_state = self.sh.inv_transform(self.phi_s_lm)
        else:
            self.phi_s_lm = torch.zeros((n, n), dtype=torch.complex128, device=dev)
            self.phi_s_anom_lm = torch.zeros((n, n), dtype=torch.complex128, device=dev)
            self.surface_elevation_extrema = (0.0, 0.0)
            self._phi_s_state = None

    def forcing_ptr(self):
        return None if self.forcing is None else self.forcing.data_ptr()

    # -- Helmholtz / winds -------------------------------------------------
    def _inv_laplacian(self, coeffs):
        return spectral_op(_lib.SOP_INV_LAPLACIAN_ZERO, self.R, coeffs)

    def helmholtz(self, state: ShallowWaterState):
        return self._inv_laplacian(state.coeffs[ZETA]), self._inv_laplacian(state.coeffs[DELTA])

    def wind_on_state_grid(self, state: ShallowWaterState):
        psi, chi = self.helmholtz(state)
        uv = winds(self._state_plan.id, self.R, psi, chi)
        return uv[0], uv[1]

    def surface_geopotential_on_state_grid(self):
        """phi_s on the state sampling, or None for a flat bottom (:327-334)."""
        return self._phi_s_state

    # -- tendencies ----------------------------------------------------------
    def tendency(self, coeffs: torch.Tensor) -> torch.Tensor:
        """d/dt of the (..., 3, L+1, L+1) stack, shallow_water.py:347-418."""
        return swe_tendency(self._plan.id, self.R, self.Omega, self.gravity, self.mean_depth, self.nu4, coeffs,
                            self.forcing)

    def tendency_state(self, state: ShallowWaterState) -> ShallowWaterState:
        return ShallowWaterState(self.tendency(state.coeffs))

    def rk4(self, coeffs: torch.Tensor, dt: float, nsteps: int = 1, check: bool = True):
        """nsteps fused RK4 steps.  Stage states are checked on the product
        grid on the device; with ``check`` the bits are read once at the end
        and a violation raises ShallowWaterStateError."""
        y, status = swe_rk4(self._plan.id, self.R, self.Omega, self.gravity, self.mean_depth, self.nu4, coeffs,
                            float(dt), int(nsteps), self.forcing)
        if check:
            bits = _or_bits(status)
            if bits:
                raise ShallowWaterStateError(self._describe_bits(bits, "during RK4 stages"))
        return y

    def rk4_host(self, host_coeffs: torch.Tensor, dt: float, nsteps: int = 1, *, chunks: int = 2,
                 out: torch.Tensor | None = None, check: bool = True) -> torch.Tensor:
        """nsteps fused RK4 steps of a host-resident (preferably pinned)
        ensemble [B, 3, L+1, L+1]; the result lands in ``out`` (pinned host
        memory, allocated when None).  The members are independent, so they
        are split into ``chunks`` groups, each copied to the device, stepped
        and copied back on a CUDA stream of its own: one group's copies run on
        the copy engines while another group's steps run on the SMs.  The
        caller's current stream waits for every group.  With ``check`` the
        status bits of all groups are read once at the end."""
        if host_coeffs.is_cuda:
            raise ValueError("rk4_host takes a host tensor (use rk4 for device-resident states)")
        B = host_coeffs.shape[0]
        if out is None:
            out = torch.empty_like(host_coeffs).pin_memory()
        dev = self.sh.weights.device
        chunks = max(1, min(int(chunks), B))
        cur = torch.cuda.current_stream(dev)
        streams = getattr(self, "_host_streams", None)
        if streams is None or len(streams) < chunks:
            streams = self._host_streams = [torch.cuda.Stream(dev) for _ in range(chunks)]
        statuses = []
        edges = [B * k // chunks for k in range(chunks + 1)]
        for k in range(chunks):
            a, b = edges[k], edges[k + 1]
            if a == b:
                continue
            s = streams[k]
            s.wait_stream(cur)
            with torch.cuda.stream(s):
                d = host_coeffs[a:b].to(dev, non_blocking=True)  # stepped in place: no second device copy
                status = swe_rk4_inplace(self._plan.id, self.R, self.Omega, self.gravity, self.mean_depth, self.nu4,
                                         d, float(dt), int(nsteps), self.forcing)
                out[a:b].copy_(d, non_blocking=True)
                statuses.append(status)
            for t in (d, status):
                t.record_stream(s)
        for k in range(chunks):
            cur.wait_stream(streams[k])
        if check:
            bits = _or_bits(torch.cat(statuses)) if statuses else 0
            if bits:
                raise ShallowWaterStateError(self._describe_bits(bits, "during RK4 stages"))
        return out

    def autotune(self, coeffs: torch.Tensor, dt: float, reps: int = 3) -> dict:
        """Pick the product plan's launch shapes for this batch by timing one
        RK4 step per candidate with CUDA events (results are bitwise
        independent of the shapes).  Returns {knobs: ms per step}."""
        plan = self._plan
        split = getattr(plan, "precision", _lib.PREC_FP64) == _lib.PREC_SPLIT_BF16
        base = list(plan.tuning())
        stream = torch.cuda.current_stream(coeffs.device)

        def time_knobs(knobs):
            plan.set_tuning(knobs)
            self.rk4(coeffs, dt, 1, check=False)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                self.rk4(coeffs, dt, 1, check=False)
            b.record(stream)
            b.synchronize()
            return a.elapsed_time(b) / reps

        results = {}
        best = list(base)
        best_ms = time_knobs(best)
        results[tuple(best)] = best_ms
        B = coeffs.reshape(-1, 3, self.l_max + 1, self.l_max + 1).shape[0]
        # knob 2: row-stage threads; 0/1: FP64 Legendre members per CTA;
        # 3/4: split synthesis / analysis slicing members per CTA
        choices = [(2, (128, 192, 256))] + ([(3, (1, 2, 4, 8)), (4, (1, 2, 4, 8))] if split
                                            else [(0, (1, 2, 3, 4)), (1, (1, 2, 3, 4))])
        for idx, cands in choices:
            for c in cands:
                if idx != 2 and c > B:
                    continue
                knobs = list(best)
                knobs[idx] = c
                ms = time_knobs(knobs)
                results[tuple(knobs)] = ms
                if ms < best_ms:
                    best, best_ms = knobs, ms
        plan.set_tuning(best)
        return {"chosen": tuple(best), "ms_per_step": best_ms, "timed": {str(k): v for k, v in results.items()}}

    # -- validation ----------------------------------------------------------
    def _validate_raw(self, coeffs):
        return swe_validate(self._state_plan.id, self._plan.id, self.R, self.Omega, self.gravity,
                            self.mean_depth, coeffs)

    def total_geopotential_extrema(self, state: ShallowWaterState):
        """(min, max) of Phi0 + phi over the state and product samplings."""
        _, ext = self._validate_raw(state.coeffs)
        e = ext.reshape(-1, 2)[0].tolist()
        return e[0], e[1]

    def characteristic_fields(self, state: ShallowWaterState) -> dict:
        u, v = self.wind_on_state_grid(state)
        wind = torch.sqrt(u * u + v * v)
        phi_total = self.phi0 + self.sh.inv_transform(state.coeffs[PHI])
        return {"u": u, "v": v, "wind_speed": wind, "phi_total": phi_total,
                "phi_total_extrema": self.total_geopotential_extrema(state)}

    def max_characteristic_speed(self, state: ShallowWaterState) -> float:
        f = self.characteristic_fields(state)
        _, phi_max = f["phi_total_extrema"]
        return float(f["wind_speed"].max()) + math.sqrt(max(phi_max, 0.0))

    def _describe_bits(self, bits: int, where: str) -> str:
        parts = []
        if bits & _lib.STATE_NONFINITE:
            parts.append("shallow-water state contains NaN/Inf coefficients")
        if bits & _lib.STATE_MONOPOLE:
            parts.append("a monopole (zeta, delta or phi a00) is nonzero; the global mean must stay exactly zero")
        if bits & _lib.STATE_THICKNESS:
            terrain = ""
            if self.has_topography:
                terrain = (f" (bottom topography {self.topography.describe()}, max surface elevation "
                           f"{self.surface_elevation_extrema[1]:g} m vs mean fluid thickness {self.mean_depth:g} m "
                           "— the terrain may protrude through the fluid layer)")
            parts.append(f"fluid thickness is not strictly positive (min(Phi0 + phi) <= 0, Phi0 = {self.phi0:g}); "
                         f"the fluid depth has collapsed{terrain}")
        return "; ".join(parts) + (f" {where}" if where else "")

    def validate_state(self, state: ShallowWaterState, *, context: str = "") -> None:
        """Raise ShallowWaterStateError on a violated constraint, :494-539."""
        status, ext = self._validate_raw(state.coeffs)
        bits = _or_bits(status)
        if bits:
            msg = self._describe_bits(bits, context)
            if bits & _lib.STATE_THICKNESS:
                msg += f" (min(Phi0 + phi) = {float(ext.reshape(-1, 2)[:, 0].min()):g} m^2/s^2)"
            raise ShallowWaterStateError(msg)

    # -- diagnostics -------------------------------------------------------
    def invariants(self, state: ShallowWaterState) -> dict:
        """Spectral mass, quadrature energy and L2 norms (run/swe/diagnostics.py:76-173)."""
        out = swe_invariants(self._state_plan.id, self.R, self.Omega, self.gravity, self.mean_depth, state.coeffs)
        keys = ("total_mass", "total_energy", "zeta_l2", "delta_l2", "phi_l2")
        vals = out.reshape(-1, 5)[0].tolist()
        return dict(zip(keys, vals))
