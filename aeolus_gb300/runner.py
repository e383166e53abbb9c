"""Run driver for ``aeolus run bve|swe`` on the GB300 models.

What a run does around the device step, with the reference's contracts:

* snapshot schedules, the advective CFL ceiling and the step/store scheduler
  of src/planetary_sandbox/run/engine.py:59-405 (count mode lands exactly on
  every target; interval mode keeps the historical countdown with its
  1e-6 * dt_snapshots tolerance; the ceiling is recomputed from every
  accepted state's characteristic speed);
* the per-step diagnostics rows of run/bve/diagnostics.py:34-220 and
  run/swe/diagnostics.py:52-173 (``diagnostics/timeseries.csv``, flushed per
  row; BVE degree spectra in ``diagnostics/spectra.npz``);
* the run capsule arrays of run/bve/runner.py:180-190 and
  run/swe/runner.py:120-127 (``vorticity_coeffs.npy``, ``vorticity_grid.npy``,
  ``bve_snapshot_times.npy``; ``swe_coeffs.npy``, ``swe_snapshot_times.npy``).

Each accepted step is one fused RK4 step on the device (``model.rk4``): the
four tendency chains and the stage updates run as library kernels, and the
shallow-water stage states are checked on the device (NaN/Inf, monopoles,
fluid thickness) with one status read per step.  Figures are not produced:
plotting is not part of this package, so a run writes the data products
only and says so once when figures were asked for.
"""
from __future__ import annotations

import csv
import math
import pathlib
import warnings
from typing import Optional, Sequence

import numpy as np
import torch

SECONDS_PER_DAY = 86400.0
CFL_NUMBER = 0.5
DEFAULT_CFL_FALLBACK_SECONDS = 600.0
BVE_SNAPSHOT_TIMES_FILENAME = "bve_snapshot_times.npy"

BVE_CSV_COLUMNS = ["time_s", "dt_s", "step", "max_speed_ms", "cfl", "circulation", "energy",
                   "enstrophy_rel", "enstrophy_abs", "zeta_max", "zeta_rms", "energy_l1",
                   "high_l_enstrophy_frac", "roundtrip_residual"]
SWE_CSV_COLUMNS = ["time_s", "dt_s", "step", "max_wind_ms", "max_char_speed_ms", "cfl", "phi_total_min",
                   "phi_total_max", "total_mass", "total_energy", "h_min_m", "eta_min_m", "eta_max_m",
                   "terrain_max_m", "zeta_l2", "delta_l2", "phi_l2"]


# ------------------------------------------------------------------ schedules
def _finite(name: str, value) -> float:
    try:
        x = float(value)
    except (TypeError, ValueError):
        raise ValueError(f"{name} must be a real number, got {value!r}") from None
    if not math.isfinite(x):
        raise ValueError(f"{name} must be finite, got {x}")
    return x


def interval_snapshot_times(dt_snapshots: float, t_end: float) -> list[float]:
    """t = 0 and every interval boundary up to t_end (1e-6 * dt tolerance),
    engine.py:59-73."""
    tol = 1e-6 * dt_snapshots
    n = 0
    out = []
    while n * dt_snapshots <= t_end + tol:
        out.append(min(n * dt_snapshots, t_end))
        n += 1
    return out


def count_snapshot_times(n_snapshots: int, t_end: float) -> list[float]:
    """N evenly spaced times with both endpoints exact, engine.py:76-89."""
    if n_snapshots <= 0:
        return []
    if n_snapshots == 1:
        return [t_end]
    h = t_end / (n_snapshots - 1)
    out = [k * h for k in range(n_snapshots - 1)]
    out.append(t_end)
    return out


def advective_cfl_timestep(length_scale: Optional[float], max_speed: float, *,
                           cfl_number: float = CFL_NUMBER,
                           fallback: float = DEFAULT_CFL_FALLBACK_SECONDS) -> float:
    """cfl_number * L / max_speed, or ``fallback`` without a length scale or
    for a motionless state; NaN/inf/negative inputs raise (engine.py:103-136)."""
    speed = _finite("max_speed", max_speed)
    if speed < 0:
        raise ValueError(f"max_speed must be >= 0, got {speed}")
    if length_scale is None:
        return fallback
    scale = _finite("length_scale", length_scale)
    if scale < 0:
        raise ValueError(f"length_scale must be >= 0, got {scale}")
    if scale == 0.0 or speed == 0.0:
        return fallback
    dt = cfl_number * scale / speed
    if not (math.isfinite(dt) and dt > 0.0):
        raise ValueError(f"advective CFL timestep is not finite and positive (got {dt} from "
                         f"length_scale={scale}, max_speed={speed}, cfl_number={cfl_number})")
    return dt


def validate_snapshot_schedule(times: Sequence[float], t_end: float) -> list[float]:
    """Finite, strictly increasing times inside [0, t_end] (a 1e-9 relative
    slack at the ends is clipped), engine.py:375-399."""
    if not (math.isfinite(t_end) and t_end > 0):
        raise ValueError(f"t_end must be finite and positive, got {t_end}")
    slack = max(1e-9, 1e-9 * t_end)
    out: list[float] = []
    for k, t in enumerate(times):
        if not math.isfinite(t):
            raise ValueError(f"snapshot_times[{k}] = {t} is not finite")
        if t < -slack or t > t_end + slack:
            raise ValueError(f"snapshot_times[{k}] = {t} is outside [0, {t_end}]")
        c = min(t_end, max(0.0, float(t)))
        if out and c <= out[-1]:
            raise ValueError(f"snapshot_times must be strictly increasing without duplicates; got {times!r}")
        out.append(c)
    return out


class IntegrationScheduler:
    """Step/store events one at a time, each step sized against the ceiling
    passed with the call that returns it (engine.py:236-305).

    Events are ``("store", 0.0, t)`` or ``("step", dt, t_after)``; ``None``
    ends the run.  Count mode stores every target once reached (no tolerance:
    a positive residual gets its own step), clips steps to land exactly on
    the next target or t_end and refuses steps that cannot advance the clock.
    Interval mode stores at t = 0 and whenever the countdown to the next
    boundary falls within 1e-6 * dt_snapshots, and stops once the remaining
    time is within that tolerance.
    """

    def __init__(self, t_end: float, *, mode: str, snapshot_times: Optional[Sequence[float]] = None,
                 dt_snapshots: Optional[float] = None):
        self.mode = mode
        self.t_end = float(t_end)
        self.t = 0.0
        self._done = False
        if mode == "count":
            self._targets = [float(x) for x in (snapshot_times or [])]
            self._next = 0
        elif mode == "interval":
            if dt_snapshots is None:
                raise ValueError("interval mode requires dt_snapshots")
            self._dts = float(dt_snapshots)
            self._tol = 1e-6 * self._dts
            self._countdown = 0.0
            self._at_top = True
        else:
            raise ValueError(f"unknown integration mode: {mode!r}")

    def next_event(self, dt_cfl: float):
        if not (math.isfinite(dt_cfl) and dt_cfl > 0):
            raise ValueError(f"dt_cfl must be finite and positive, got {dt_cfl}")
        if self._done:
            return None
        ev = self._count_event(dt_cfl) if self.mode == "count" else self._interval_event(dt_cfl)
        if ev is None:
            self._done = True
        return ev

    def _count_event(self, dt_cfl: float):
        tg = self._targets
        if self._next < len(tg) and tg[self._next] <= self.t:
            self._next += 1
            return ("store", 0.0, tg[self._next - 1])
        if self._next >= len(tg) and self.t >= self.t_end:
            return None
        stop = tg[self._next] if self._next < len(tg) else self.t_end
        gap = stop - self.t
        if gap <= 0.0:
            raise RuntimeError(f"count planner expected a positive residual, got {gap} at t={self.t} "
                               f"for target={stop}")
        if dt_cfl >= gap:
            self.t = stop
            return ("step", gap, stop)
        t_new = self.t + dt_cfl
        if t_new <= self.t:
            raise FloatingPointError(f"count planner step stagnated at t={self.t}: dt_cfl={dt_cfl} "
                                     f"cannot advance time toward target={stop}")
        if t_new > stop:
            raise FloatingPointError(f"count planner step overshot target={stop}: t={self.t}, dt={dt_cfl}, "
                                     f"t_after={t_new}")
        self.t = t_new
        return ("step", dt_cfl, t_new)

    def _interval_event(self, dt_cfl: float):
        if self._at_top:
            if not self.t <= self.t_end + self._tol:
                return None
            self._at_top = False
            if self._countdown <= self._tol:
                self._countdown = self._dts
                return ("store", 0.0, self.t)
        remaining = self.t_end - self.t
        if remaining <= self._tol:
            return None
        dt = min(dt_cfl, self._countdown, remaining)
        if dt <= 0:
            return None
        self.t += dt
        self._countdown = max(0.0, self._countdown - dt)
        self._at_top = True
        return ("step", dt, self.t)


def integration_plan(t_end: float, dt_cfl: float, *, mode: str, snapshot_times=None, dt_snapshots=None):
    """All events for a constant ceiling (engine.py:308-334)."""
    if not (math.isfinite(dt_cfl) and dt_cfl > 0):
        raise ValueError(f"dt_cfl must be finite and positive, got {dt_cfl}")
    sch = IntegrationScheduler(t_end, mode=mode, snapshot_times=snapshot_times, dt_snapshots=dt_snapshots)
    events = []
    while (ev := sch.next_event(dt_cfl)) is not None:
        events.append(ev)
    return events


def integrate(scheduler: IntegrationScheduler, dt_cfl: float, length_scale: Optional[float], *,
              on_step, on_store) -> tuple[float, int]:
    """Drive the scheduler; after each accepted step the ceiling comes from
    that step's characteristic speed (engine.py:402-431 loop contract).
    ``on_step(t_before, t_after, dt, step) -> max speed``; returns (t, steps)."""
    t, step = 0.0, 0
    while (ev := scheduler.next_event(dt_cfl)) is not None:
        kind, dt, t_ev = ev
        if kind == "store":
            on_store(t_ev)
            continue
        step += 1
        speed = on_step(t, t_ev, dt, step)
        t = t_ev
        dt_cfl = advective_cfl_timestep(length_scale, speed)
    return t, step


def _resolve_schedule(snapshot_mode, snapshot_times, dt_snapshots, t_end):
    if snapshot_mode is None:
        snapshot_mode = "interval" if snapshot_times is None else "count"
    if snapshot_mode not in ("count", "interval"):
        raise ValueError(f"unknown snapshot_mode: {snapshot_mode!r}")
    if snapshot_mode == "count":
        if snapshot_times is None:
            raise ValueError("count mode requires an explicit snapshot_times schedule")
        snapshot_times = validate_snapshot_schedule(snapshot_times, t_end)
    elif dt_snapshots is None:
        raise ValueError("interval mode requires dt_snapshots")
    return snapshot_mode, snapshot_times


def _no_figures(plots):
    if plots is None or len(tuple(plots)) > 0:
        warnings.warn("figures are not rendered by aeolus_gb300 (plotting is outside this package); "
                      "the run writes its data products only", stacklevel=3)


class _CsvRows:
    def __init__(self, out_dir: pathlib.Path, columns):
        self.dir = pathlib.Path(out_dir) / "diagnostics"
        self.dir.mkdir(parents=True, exist_ok=True)
        self._f = open(self.dir / "timeseries.csv", "w", newline="", encoding="utf-8")
        self._w = csv.DictWriter(self._f, fieldnames=columns)
        self._w.writeheader()

    def write(self, row: dict):
        self._w.writerow(row)
        self._f.flush()

    def close(self):
        if not self._f.closed:
            self._f.close()


# ------------------------------------------------------------------ BVE run
def _degree_power(c: torch.Tensor) -> torch.Tensor:
    """Per-degree power P_l = Re(a_l0)^2 + 2 sum_{0<m<=l} |a_lm|^2."""
    n = c.shape[-1]
    lm = torch.arange(n, device=c.device)
    p = torch.where(lm[None, :] == 0, c.real ** 2, 2.0 * (c.real ** 2 + c.imag ** 2))
    p = torch.where(lm[None, :] <= lm[:, None], p, torch.zeros((), dtype=p.dtype, device=p.device))
    return p.sum(dim=1)


class DiagnosticsRecorder:
    """BVE rows (run/bve/diagnostics.py:127-220): spectral invariants from the
    library's reduction kernel, zeta max/rms on the state grid, max |u| from
    the streamfunction winds, the transform round-trip residual and degree
    spectra every ``roundtrip_every`` / ``spectra_every`` records."""

    def __init__(self, sh, so, grid, radius: float, omega: float, out_dir, spectra_every: int = 10,
                 roundtrip_every: int = 10):
        self.sh, self.so, self.grid = sh, so, grid
        self.R, self.omega = float(radius), float(omega)
        self.spectra_every, self.roundtrip_every = int(spectra_every), int(roundtrip_every)
        self.min_edge = getattr(grid, "cfl_length_scale", None)
        self._csv = _CsvRows(out_dir, BVE_CSV_COLUMNS)
        self.dir = self._csv.dir
        self._n = 0
        self._spec_t, self._spec_E, self._spec_Z = [], [], []

    def record(self, t: float, zeta_lm: torch.Tensor, dt: float, step: int) -> dict:
        from .diagnostics import spectral_diagnostics

        spec = spectral_diagnostics(zeta_lm, self.R, self.omega)
        zeta = self.sh.inv_transform(zeta_lm)
        w = self.sh.weights
        u, v = self.so.velocity_from_streamfunction(self.so.inv_laplacian(zeta_lm))
        vals = [zeta.abs().max(), torch.sqrt(torch.sum(w * zeta.reshape(w.shape) ** 2) / torch.sum(w)),
                torch.sqrt(u * u + v * v).max()]
        roundtrip = float("nan")
        if self.roundtrip_every > 0 and self._n % self.roundtrip_every == 0:
            back = self.sh.transform(zeta)
            vals += [torch.linalg.norm(back - zeta_lm), torch.linalg.norm(zeta_lm)]
        host = torch.stack([x.to(torch.float64) for x in vals]).tolist()
        if len(host) == 5:
            roundtrip = host[3] / (host[4] + 1e-300)
        max_speed = host[2]
        row = {"time_s": t, "dt_s": dt, "step": step, "max_speed_ms": max_speed,
               "cfl": (max_speed * dt / self.min_edge) if (self.min_edge and dt > 0) else float("nan"),
               "circulation": spec["circulation"], "energy": spec["energy"],
               "enstrophy_rel": spec["enstrophy_rel"], "enstrophy_abs": spec["enstrophy_abs"],
               "zeta_max": host[0], "zeta_rms": host[1], "energy_l1": spec["energy_l1"],
               "high_l_enstrophy_frac": spec["high_l_enstrophy_frac"], "roundtrip_residual": roundtrip}
        self._csv.write(row)
        if self.spectra_every > 0 and self._n % self.spectra_every == 0:
            P = _degree_power(zeta_lm)
            L = zeta_lm.shape[-1] - 1
            l = torch.arange(L + 1, dtype=torch.float64, device=P.device)
            inv = torch.zeros_like(l)
            inv[1:] = 1.0 / (l[1:] * (l[1:] + 1.0))
            self._spec_t.append(t)
            self._spec_E.append((0.5 * self.R ** 4 * inv * P).cpu().numpy())
            self._spec_Z.append((0.5 * self.R ** 2 * P).cpu().numpy())
        self._n += 1
        return row

    def close(self):
        if self._spec_t:
            np.savez(self.dir / "spectra.npz", times=np.asarray(self._spec_t),
                     energy_l=np.asarray(self._spec_E), enstrophy_l=np.asarray(self._spec_Z))
        self._csv.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_bve(planet, zeta0_lm, dt_snapshots: float | None, t_end_days: float, out_dir, viscosity: float,
            scenario: str = "two_vortices", figure_metadata: dict | None = None,
            snapshot_times: Sequence[float] | None = None, plots: Sequence[str] | None = None,
            snapshot_mode: str | None = None) -> int:
    """Integrate the BVE with state-adaptive CFL steps and write the run
    capsule (run/bve/runner.py:33-190): vorticity coefficient and grid
    snapshot stacks, stored times, diagnostics rows and spectra."""
    from .barotropic import BarotropicState, BarotropicVorticity

    out_dir = pathlib.Path(out_dir)
    model = BarotropicVorticity(planet, scenario=scenario, viscosity=viscosity)
    t_end = t_end_days * SECONDS_PER_DAY
    snapshot_mode, snapshot_times = _resolve_schedule(snapshot_mode, snapshot_times, dt_snapshots, t_end)
    _no_figures(plots)
    dev = planet.sh.weights.device
    state = BarotropicState(torch.as_tensor(zeta0_lm, dtype=torch.complex128, device=dev).clone())
    length_scale = getattr(planet.grid, "cfl_length_scale", None)
    zeta_initial_grid = planet.sh.inv_transform(state.coeffs)
    recorder = DiagnosticsRecorder(planet.sh, planet.so, planet.grid, planet.params.radius,
                                   planet.params.angular_velocity, out_dir)
    first = recorder.record(0.0, state.coeffs, dt=0.0, step=0)
    dt_cfl = advective_cfl_timestep(length_scale, first["max_speed_ms"])
    coeff_snaps, grid_snaps, stored = [], [], []
    step = 0

    def on_store(t_ev: float):
        coeff_snaps.append(state.coeffs.cpu().numpy())
        stored.append(t_ev)
        grid_snaps.append(planet.sh.inv_transform(state.coeffs).cpu().numpy())
        print(f"Time: {t_ev / 3600.0:8.2f} hrs | Step: {step} ")

    def on_step(t0: float, t1: float, dt: float, k: int) -> float:
        nonlocal state, step
        state = BarotropicState(model.rk4(state.coeffs, dt, 1))
        step = k
        return recorder.record(t1, state.coeffs, dt=dt, step=k)["max_speed_ms"]

    sch = IntegrationScheduler(t_end, mode=snapshot_mode, snapshot_times=snapshot_times,
                               dt_snapshots=dt_snapshots)
    try:
        integrate(sch, dt_cfl, length_scale, on_step=on_step, on_store=on_store)
    finally:
        recorder.close()
    if coeff_snaps:
        coeffs_stack, grid_stack = np.stack(coeff_snaps), np.stack(grid_snaps)
    else:
        coeffs_stack = np.empty((0, *state.coeffs.shape), dtype=np.complex128)
        grid_stack = np.empty((0, *zeta_initial_grid.shape), dtype=np.float64)
    np.save(out_dir / "vorticity_coeffs.npy", coeffs_stack)
    np.save(out_dir / "vorticity_grid.npy", grid_stack)
    np.save(out_dir / BVE_SNAPSHOT_TIMES_FILENAME, np.asarray(stored, dtype=np.float64))
    return 0


# ------------------------------------------------------------------ SWE run
class SWEDiagnosticsRecorder:
    """Shallow-water rows (run/swe/diagnostics.py:90-173): winds and total
    geopotential on the state grid, extrema over the state and product
    samplings from the library's validation kernel, spectral mass,
    quadrature energy and L2 norms from its invariant kernel, plus the
    topographic terms of the energy and free-surface anomaly over terrain."""

    def __init__(self, model, out_dir):
        self.model = model
        self.R = model.R
        self.length_scale = getattr(model.grid, "cfl_length_scale", None)
        self._csv = _CsvRows(out_dir, SWE_CSV_COLUMNS)
        self.dir = self._csv.dir

    def record(self, t: float, state, dt: float, step: int) -> dict:
        m = self.model
        f = m.characteristic_fields(state)
        phi_min, phi_max = f["phi_total_extrema"]
        phi_s = m.surface_geopotential_on_state_grid()
        if phi_s is None:
            eta = (f["phi_total"] - m.phi0) / m.gravity
            topo_energy = torch.zeros((), dtype=torch.float64, device=eta.device)
        else:
            # free-surface anomaly and the topographic potential energy Phi phi_s
            mean_phi_s = float(m.phi_s_lm[0, 0].real) / math.sqrt(4.0 * math.pi)
            eta = (f["phi_total"] - m.phi0 + (phi_s - mean_phi_s)) / m.gravity
            topo_energy = torch.sum(m.sh.weights * self.R ** 2 * f["phi_total"] * phi_s)
        w_max, e_min, e_max, e_topo = torch.stack([f["wind_speed"].max(), eta.min(), eta.max(),
                                                   topo_energy]).tolist()
        inv = m.invariants(state)
        inv["total_energy"] += e_topo
        max_char = w_max + math.sqrt(max(phi_max, 0.0))
        row = {"time_s": t, "dt_s": dt, "step": step, "max_wind_ms": w_max, "max_char_speed_ms": max_char,
               "cfl": (max_char * dt / self.length_scale) if (self.length_scale and dt > 0) else float("nan"),
               "phi_total_min": phi_min, "phi_total_max": phi_max, "total_mass": inv["total_mass"],
               "total_energy": inv["total_energy"], "h_min_m": phi_min / m.gravity, "eta_min_m": e_min,
               "eta_max_m": e_max, "terrain_max_m": m.surface_elevation_extrema[1],
               "zeta_l2": inv["zeta_l2"], "delta_l2": inv["delta_l2"], "phi_l2": inv["phi_l2"]}
        self._csv.write(row)
        return row

    def close(self):
        self._csv.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_swe(model, state0, dt_snapshots: float | None, t_end_days: float, out_dir,
            figure_metadata: dict | None = None, snapshot_times: Sequence[float] | None = None,
            plots: Sequence[str] | None = None, snapshot_mode: str | None = None, scenario: str = "swe") -> int:
    """Integrate the shallow-water equations and write the run capsule
    (run/swe/runner.py:29-127).  Every accepted step is validated (stage
    states on the device inside the fused step, the accepted state by the
    validation kernel); a violation raises ShallowWaterStateError and the
    diagnostics written so far stay on disk."""
    from .shallow_water import ShallowWaterState

    out_dir = pathlib.Path(out_dir)
    t_end = t_end_days * SECONDS_PER_DAY
    snapshot_mode, snapshot_times = _resolve_schedule(snapshot_mode, snapshot_times, dt_snapshots, t_end)
    _no_figures(plots)
    model.validate_state(state0, context="initial state")
    dev = model.sh.weights.device
    state = ShallowWaterState(torch.as_tensor(state0.coeffs, dtype=torch.complex128, device=dev).clone())
    length_scale = getattr(model.planet.grid, "cfl_length_scale", None)
    recorder = SWEDiagnosticsRecorder(model, out_dir)
    first = recorder.record(0.0, state, dt=0.0, step=0)
    dt_cfl = advective_cfl_timestep(length_scale, first["max_char_speed_ms"])
    snaps, stored = [], []
    step = 0

    def on_store(t_ev: float):
        snaps.append(state.coeffs.cpu().numpy())
        stored.append(t_ev)
        print(f"Time: {t_ev / 3600.0:8.2f} hrs | Step: {step} ")

    def on_step(t0: float, t1: float, dt: float, k: int) -> float:
        nonlocal state, step
        try:
            state = ShallowWaterState(model.rk4(state.coeffs, dt, 1))
        except ValueError as err:
            raise type(err)(f"{err} (in an RK4 stage after step {step})") from None
        step = k
        model.validate_state(state, context=f"at t={t1:g} s (step {k})")
        return recorder.record(t1, state, dt=dt, step=k)["max_char_speed_ms"]

    sch = IntegrationScheduler(t_end, mode=snapshot_mode, snapshot_times=snapshot_times,
                               dt_snapshots=dt_snapshots)
    try:
        integrate(sch, dt_cfl, length_scale, on_step=on_step, on_store=on_store)
    finally:
        recorder.close()
    stack = np.stack(snaps) if snaps else np.empty((0, *state.coeffs.shape), dtype=np.complex128)
    np.save(out_dir / "swe_coeffs.npy", stack)
    np.save(out_dir / "swe_snapshot_times.npy", np.asarray(stored, dtype=np.float64))
    return 0


# ------------------------------------------------------------------ PE run
PE_CSV_COLUMNS = ["time_s", "dt_s", "step", "t_min", "t_max", "ps_min", "ps_max", "max_wind_ms", "max_abs_zeta",
                  "max_abs_delta", "max_char_speed_ms", "courant", "total_mass", "mass_rel_drift"]


class PEDiagnosticsRecorder:
    """Primitive-equation rows (run/pe/diagnostics.py:62-140): temperature
    extrema over both samplings, surface-pressure extrema, winds, zeta and
    delta maxima on the state grid, the characteristic speed, a diagnostic
    Courant number and the quadrature mass with its drift from the first
    row."""

    def __init__(self, model, out_dir):
        self.model = model
        self.R = model.R
        self.length_scale = getattr(model.grid, "cfl_length_scale", None)
        self._csv = _CsvRows(out_dir, PE_CSV_COLUMNS)
        self.dir = self._csv.dir
        self._mass0 = None

    def record(self, t: float, state, dt: float, step: int) -> dict:
        from .ops import synthesize

        m = self.model
        t_min, t_max = m.temperature_extrema(state)
        ps = m.surface_pressure_on_state_grid(state)
        u, v = m.wind_on_state_grid(state)
        zd = synthesize(m.sh.plan.id, state.coeffs[:2 * m.nlev])
        mass_t = torch.sum(m.sh.weights * self.R ** 2 * ps)
        vals = torch.stack([ps.min(), ps.max(), torch.sqrt(u * u + v * v).max(), zd[:m.nlev].abs().max(),
                            zd[m.nlev:].abs().max(), mass_t]).tolist()
        max_char = m.max_characteristic_speed(state)
        total_mass = vals[5]
        if self._mass0 is None:
            self._mass0 = total_mass
        row = {"time_s": t, "dt_s": dt, "step": step, "t_min": t_min, "t_max": t_max, "ps_min": vals[0],
               "ps_max": vals[1], "max_wind_ms": vals[2], "max_abs_zeta": vals[3], "max_abs_delta": vals[4],
               "max_char_speed_ms": max_char,
               "courant": (max_char * dt / self.length_scale) if (self.length_scale and dt > 0) else float("nan"),
               "total_mass": total_mass,
               "mass_rel_drift": (total_mass - self._mass0) / self._mass0 if self._mass0 else 0.0}
        self._csv.write(row)
        return row

    def close(self):
        self._csv.close()


def run_pe(model, state0, *, dt_seconds: float, t_end_days: float, out_dir, snapshot_times: Sequence[float],
           snapshot_mode: str = "count", dt_snapshots: float | None = None, figure_metadata: dict | None = None,
           plots: Sequence[str] | None = None, scenario: str = "pe") -> int:
    """Fixed-step primitive-equation run (run/pe/runner.py:48-165): the
    scheduler driven with a constant ceiling (steps clipped only to land on
    output times and t_end), every RK4 stage and accepted state validated,
    a diagnostics row per step, ``pe_coeffs.npy`` and ``pe_snapshot_times.npy``."""
    from .engine import rk4_step_array
    from .primitive_equations import PrimitiveEquationsState

    out_dir = pathlib.Path(out_dir)
    t_end = t_end_days * SECONDS_PER_DAY
    if not (math.isfinite(dt_seconds) and dt_seconds > 0):
        raise ValueError(f"dt_seconds must be finite and > 0, got {dt_seconds}")
    if snapshot_mode not in ("count", "interval"):
        raise ValueError(f"unknown snapshot_mode: {snapshot_mode!r}")
    _no_figures(plots)
    model.validate_state(state0, context="initial state")
    dev = model.phi_surface_lm.device
    state = PrimitiveEquationsState(torch.as_tensor(state0.coeffs, dtype=torch.complex128, device=dev).clone())
    recorder = PEDiagnosticsRecorder(model, out_dir)
    last = recorder.record(0.0, state, dt=0.0, step=0)
    snaps, stored = [], []
    step = 0

    def validate_stage(y):
        model.validate_state(PrimitiveEquationsState(y), context=f"in an RK4 stage after step {step}")

    sch = IntegrationScheduler(t_end, mode=snapshot_mode, snapshot_times=snapshot_times, dt_snapshots=dt_snapshots)
    try:
        t = 0.0
        while (ev := sch.next_event(dt_seconds)) is not None:
            kind, dt, t_ev = ev
            if kind == "store":
                snaps.append(state.coeffs.cpu().numpy())
                stored.append(t_ev)
                print(f"Time: {t_ev / 3600.0:8.3f} hrs | Step: {step} ")
                continue
            # `step` still names the last accepted step while the stages run
            # (a stage fault reads "after step k-1", run/pe/runner.py:96-106)
            y = rk4_step_array(model.tendency, state.coeffs, t, dt, stage_validator=validate_stage)
            step += 1
            state = PrimitiveEquationsState(y)
            model.validate_state(state, context=f"at t={t_ev:g} s (step {step})")
            last = recorder.record(t_ev, state, dt=dt, step=step)
            t = t_ev
    finally:
        recorder.close()
    stack = np.stack(snaps) if snaps else np.empty((0, *state.coeffs.shape), dtype=np.complex128)
    np.save(out_dir / "pe_coeffs.npy", stack)
    np.save(out_dir / "pe_snapshot_times.npy", np.asarray(stored, dtype=np.float64))
    print(f"Stored {len(stored)} snapshot(s) over {step} fixed {dt_seconds:g} s step(s).")
    print(f"Final diagnostics @ t={last['time_s'] / 3600.0:.3f} h: T[min,max]=[{last['t_min']:.2f}, "
          f"{last['t_max']:.2f}] K, p_s[min,max]=[{last['ps_min']:.1f}, {last['ps_max']:.1f}] Pa, "
          f"max|V|={last['max_wind_ms']:.3g} m/s, mass drift={last['mass_rel_drift']:.2e}")
    return 0
